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

// Factorials, binomials and reciprocals come from a constant-memory table, filled by
// static initialization from a constexpr builder, in both FP64 and FP32 (each FP32
// entry is the FP64 value rounded once).  A table read is one constant-bank operand
// when the loop around it is unrolled and one constant load when it is not; no
// FP64 arithmetic is left at run time in the FP32 kernels (FP64 throughput is a small
// fraction of FP32 on this part).  The builder is iterative: a recursive device
// function has no static stack bound.
struct GxTables {
    double fact[34];
    double invfact[34];
    double binom[17][17];
    float binom_f[17][17];
    double ifp[17][17];  // 1/(i! j!) as the FP64 product of 1/i! and 1/j!
    float ifp_f[17][17];
    double inv[34];  // 1/n
    float inv_f[34];
    double ff[33][33];  // k! l! (derivative scale, k + l <= 32)
    float ff_f[33][33];
};
__host__ __device__ constexpr GxTables gx_make_tables() {
    GxTables t{};
    t.fact[0] = 1.0;
    for (int i = 1; i < 34; i++) t.fact[i] = t.fact[i - 1] * (double)i;
    for (int i = 0; i < 34; i++) t.invfact[i] = 1.0 / t.fact[i];
    for (int n = 0; n < 17; n++) {
        t.binom[n][0] = 1.0;
        for (int k = 1; k <= n; k++) t.binom[n][k] = t.binom[n - 1][k - 1] + (k < n ? t.binom[n - 1][k] : 0.0);
        for (int k = 0; k < 17; k++) t.binom_f[n][k] = (float)t.binom[n][k];
    }
    for (int i = 0; i < 17; i++)
        for (int j = 0; j < 17; j++) {
            t.ifp[i][j] = t.invfact[i] * t.invfact[j];
            t.ifp_f[i][j] = (float)t.ifp[i][j];
        }
    for (int i = 0; i < 33; i++)
        for (int j = 0; j < 33; j++) {
            t.ff[i][j] = i + j <= 32 ? t.fact[i] * t.fact[j] : 0.0;
            t.ff_f[i][j] = (float)t.ff[i][j];
        }
    t.inv[0] = 0.0;
    t.inv_f[0] = 0.f;
    for (int i = 1; i < 34; i++) {
        t.inv[i] = 1.0 / (double)i;
        t.inv_f[i] = (float)t.inv[i];
    }
    return t;
}
__constant__ GxTables c_tab = gx_make_tables();
__device__ __forceinline__ double cfact(int n) { return c_tab.fact[n]; }
__device__ __forceinline__ double cinvfact(int n) { return c_tab.invfact[n]; }
__device__ __forceinline__ double cbinom(int n, int k) { return (k < 0 || k > n) ? 0.0 : c_tab.binom[n][k]; }
// typed reads: C(n, k), 1/(i! j!), 1/n
template <class T> __device__ __forceinline__ T tab_binom(int n, int k);
template <> __device__ __forceinline__ double tab_binom<double>(int n, int k) { return c_tab.binom[n][k]; }
template <> __device__ __forceinline__ float tab_binom<float>(int n, int k) { return c_tab.binom_f[n][k]; }
template <class T> __device__ __forceinline__ T tab_ifp(int i, int j);
template <> __device__ __forceinline__ double tab_ifp<double>(int i, int j) { return c_tab.ifp[i][j]; }
template <> __device__ __forceinline__ float tab_ifp<float>(int i, int j) { return c_tab.ifp_f[i][j]; }
template <class T> __device__ __forceinline__ T tab_ff(int k, int l);
template <> __device__ __forceinline__ double tab_ff<double>(int k, int l) { return c_tab.ff[k][l]; }
template <> __device__ __forceinline__ float tab_ff<float>(int k, int l) { return c_tab.ff_f[k][l]; }
template <class T> __device__ __forceinline__ T tab_inv(int n);
template <> __device__ __forceinline__ double tab_inv<double>(int n) { return c_tab.inv[n]; }
template <> __device__ __forceinline__ float tab_inv<float>(int n) { return c_tab.inv_f[n]; }
__host__ __device__ constexpr int nc2(int q) { return (q + 1) * (q + 2) / 2; }  // entries with k+l <= q

// Loops over expansion indices are fully unrolled (coefficient arrays stay in
// registers) for orders up to 5; above that the bound is made a runtime value
// (a zero the compiler cannot see through) so the loops stay rolled and the
// translation units compile in seconds.
__constant__ int g_rt_zero = 0;
__device__ __forceinline__ int gx_rt_order(int P) { return P <= 8 ? P : P + g_rt_zero; }

template <class T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// FP32 reciprocal square root as the single PTX instruction rsqrt.approx.ftz.f32:
// the arguments here are r^2 + eps^2 > 0, far from the denormal range, so the
// denormal handling the library function adds around it is dead weight.
__device__ __forceinline__ float rsqrt_fast(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Packed FP32 pairs: the .f32x2 forms of add/sub/mul/fma (sm_100 family) issue one
// instruction for two lanes of work, each half rounded exactly as the scalar
// instruction would round it.  A pair lives in one 64-bit register (lo, hi).
__device__ __forceinline__ uint64_t pk2(float lo, float hi) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk2(uint64_t v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

template <class T>
__device__ __forceinline__ T rsqrt_t(T v);
template <>
__device__ __forceinline__ double rsqrt_t<double>(double v) { return rsqrt(v); }
template <>
__device__ __forceinline__ float rsqrt_t<float>(float v) { return rsqrt_fast(v); }

// Expansion rows are padded to a multiple of 16 bytes (16 floats / 16 doubles at
// p = 4) so that a node's coefficients load as float4 / double2 vectors.
template <class T>
__host__ __device__ constexpr int row_stride(int nc) {
    return sizeof(T) == 4 ? (nc + 3) / 4 * 4 : (nc + 1) / 2 * 2;
}

template <int N, class T>
__device__ __forceinline__ void load_row(const T *__restrict__ p, T *out);
template <int N>
__device__ __forceinline__ void load_row(const float *__restrict__ p, float *out) {
    constexpr int NS = row_stride<float>(N);
#pragma unroll
    for (int k = 0; k < NS / 4; k++) {
        float4 v = __ldg(reinterpret_cast<const float4 *>(p) + k);
        if (4 * k + 0 < N) out[4 * k + 0] = v.x;
        if (4 * k + 1 < N) out[4 * k + 1] = v.y;
        if (4 * k + 2 < N) out[4 * k + 2] = v.z;
        if (4 * k + 3 < N) out[4 * k + 3] = v.w;
    }
}
template <int N>
__device__ __forceinline__ void load_row(const double *__restrict__ p, double *out) {
    constexpr int NS = row_stride<double>(N);
#pragma unroll
    for (int k = 0; k < NS / 2; k++) {
        double2 v = __ldg(reinterpret_cast<const double2 *>(p) + k);
        if (2 * k + 0 < N) out[2 * k + 0] = v.x;
        if (2 * k + 1 < N) out[2 * k + 1] = v.y;
    }
}

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

// The same from the caller's page-locked host arrays (hx, hy, hm: their device
// addresses), read over the host link straight into the resident arrays.
__global__ void k_prepare_from(int64_t n, const double *__restrict__ hx, const double *__restrict__ hy,
                               const double *__restrict__ hm, double *x, double *y, double *m, double *ax, double *ay,
                               unsigned *status) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double xi = hx[i], yi = hy[i], mi = hm[i];
    bool bad = false;
    if (fabs(xi) > 1e100 || fabs(yi) > 1e100 || !isfinite(xi) || !isfinite(yi)) {
        xi = 0.0;
        yi = 0.0;
        bad = true;
    }
    if (!isfinite(mi) || mi <= 0.0) {
        mi = 1.0;
        bad = true;
    }
    if (bad) atomicOr(status, GX_DEV_NONFINITE_INPUT);
    x[i] = xi;
    y[i] = yi;
    m[i] = mi;
    ax[i] = 0.0;
    ay[i] = 0.0;
}

// ---------------------------------------------------------------- P2M
template <int P, class T>
__global__ void __launch_bounds__(128) k_p2m(int64_t nl, const double *__restrict__ x, const double *__restrict__ y,
                                             const double *__restrict__ m, const double *__restrict__ comx,
                                             const double *__restrict__ comy, const int32_t *__restrict__ bs,
                                             const int32_t *__restrict__ be, T *__restrict__ M,
                                             float4 *__restrict__ pos) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    (void)NCr;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (leaf >= nl) return;
    int32_t b0 = bs[leaf], b1 = be[leaf];
    double cxl = comx[leaf], cyl = comy[leaf];
    T acc[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) acc[k] = T(0);
    for (int32_t b = b0 + lane; b < b1; b += 32) {
        T dx = (T)(x[b] - cxl), dy = (T)(y[b] - cyl), mm = (T)m[b];
        if (pos) pos[b] = make_float4((float)dx, (float)dy, (float)m[b], 0.f);
        T px[P + 1], py[P + 1];
        px[0] = T(1);
        py[0] = T(1);
#pragma unroll
        for (int k = 1; k <= PP; k++) {
            px[k] = px[k - 1] * dx;
            py[k] = py[k - 1] * dy;
        }
#pragma unroll
        for (int i = 0; i <= PP; i++)
#pragma unroll
            for (int j = 0; j <= PP - i; j++)
                acc[gx_mi(i, j)] += mm * px[i] * py[j] * tab_ifp<T>(i, j);
    }
#pragma unroll
    for (int k = 0; k < NCr; k++) {
        T v = warp_sum_t<T>(acc[k]);
        if (lane == (k & 31)) M[leaf * NS + k] = isfinite(v) ? v : T(0);
    }
}

// ---------------------------------------------------------------- M2M
// One thread per parent: M_P[I,J] = sum_children sum_{i<=I, j<=J} M_c[i,j] dx^(I-i) dy^(J-j) / ((I-i)!(J-j)!)
template <int P, class T>
__global__ void __launch_bounds__(128) k_m2m(int64_t s, int64_t e, const int4 *__restrict__ child,
                                             const double *__restrict__ comx, const double *__restrict__ comy,
                                             T *__restrict__ M) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    int64_t node = s + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= e) return;
    int4 c4 = child[node];
    int cc[4] = {c4.x, c4.y, c4.z, c4.w};
    double pcx = comx[node], pcy = comy[node];
    T out[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) out[k] = T(0);
    for (int q = 0; q < 4; q++) {
        int c = cc[q];
        if (c < 0) continue;
        T dx = (T)(comx[c] - pcx), dy = (T)(comy[c] - pcy);
        T px[P + 1], py[P + 1];
        px[0] = T(1);
        py[0] = T(1);
#pragma unroll
        for (int k = 1; k <= PP; k++) {
            px[k] = px[k - 1] * dx * tab_inv<T>(k);  // dx^k / k!
            py[k] = py[k - 1] * dy * tab_inv<T>(k);
        }
        T mc[NC];
        load_row<NC>(M + (int64_t)c * NS, mc);
#pragma unroll
        for (int oi = 0; oi <= PP; oi++)
#pragma unroll
            for (int oj = 0; oj <= PP - oi; oj++)
#pragma unroll
                for (int i = 0; i <= oi; i++)
#pragma unroll
                    for (int j = 0; j <= oj; j++) out[gx_mi(oi, oj)] += mc[gx_mi(i, j)] * px[oi - i] * py[oj - j];
    }
#pragma unroll
    for (int k = 0; k < NCr; k++) M[node * NS + k] = out[k];
}

// Levels 1 .. L of single-child chains over the leaves (Morton rounds that grouped
// nothing): the level-L ancestor of leaf x is node x + L nl and holds the same bodies,
// so its moments are the leaf's shifted once to its COM (translations compose exactly);
// the chain nodes in between have no far interactions in the ACCURATE lists and their
// moments are never read.
template <int P, class T>
__global__ void __launch_bounds__(128) k_m2m_chain(int64_t nl, int64_t up, const double *__restrict__ comx,
                                                   const double *__restrict__ comy, T *__restrict__ M) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nl) return;
    const int64_t node = c + up;
    T dx = (T)(comx[c] - comx[node]), dy = (T)(comy[c] - comy[node]);
    T px[P + 1], py[P + 1];
    px[0] = T(1);
    py[0] = T(1);
#pragma unroll
    for (int k = 1; k <= PP; k++) {
        px[k] = px[k - 1] * dx * tab_inv<T>(k);
        py[k] = py[k - 1] * dy * tab_inv<T>(k);
    }
    T mc[NC], out[NC];
    load_row<NC>(M + c * NS, mc);
#pragma unroll
    for (int k = 0; k < NCr; k++) out[k] = T(0);
#pragma unroll
    for (int oi = 0; oi <= PP; oi++)
#pragma unroll
        for (int oj = 0; oj <= PP - oi; oj++)
#pragma unroll
            for (int i = 0; i <= oi; i++)
#pragma unroll
                for (int j = 0; j <= oj; j++) out[gx_mi(oi, oj)] += mc[gx_mi(i, j)] * px[oi - i] * py[oj - j];
#pragma unroll
    for (int k = 0; k < NCr; k++) M[node * NS + k] = out[k];
}

template <class T>
__global__ void k_scrub(int64_t n, T *v) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && !isfinite(v[i])) v[i] = T(0);
}

// ---------------------------------------------------------------- M2L
// Derivatives of 1/R (R^2 = dx^2+dy^2+eps^2) scaled by k! l!:  A[k,l] = k! l! a_kl with
// |k| R^2 a_k = -(2|k|-1)(dx a_{k-ex} + dy a_{k-ey}) - (|k|-1)(a_{k-2ex} + a_{k-2ey}), a_0 = 1/R.
// The recurrence runs on the unscaled a (no per-term index multipliers: two
// coefficients per order) and each term is scaled once by k! l!.
// The kernel of the reference is G = -1/R, so G^(k,l) = -A[k,l].
// One far pair, derivatives and contraction fused:  out[X] += sum_Y in[Y] A[X+Y]
// (|X|, |Y| <= p) with A the scaled derivatives at (dx, dy).  Each A[U] is used by
// every (X, Y) with X + Y = U the moment it is formed, so no derivative array is kept:
// only the unscaled values of the last two orders feed the recurrence.  The forward
// M2L takes in = signed moments (-1)^|S| M[S], out = the local accumulator; the
// adjoint M2L^T takes in = dL[T]/T!, out = the moment cotangent accumulator.
// One derivative order N of the fused M2L: the recurrence for the N+1 terms of order N
// (from the unscaled orders N-1 and N-2) and every contraction term they complete.
// A compile-time order keeps every index constant, so the arrays stay in registers.
// k! l! as a compile-time constant once the loops are unrolled
__host__ __device__ constexpr double ff_const(int k, int l) {
    double r = 1.0;
    for (int i = 2; i <= k; i++) r *= i;
    for (int i = 2; i <= l; i++) r *= i;
    return r;
}

template <int P, int N, class T>
__device__ __forceinline__ void m2l_order(T dx, T dy, T ir2, T *a, const T *in, T *out) {
    if constexpr (N <= 2 * P) {
        const T in_ = tab_inv<T>(N) * ir2;
        // c1 (dx a_{k-1,l} + dy a_{k,l-1}) + c2 (a_{k-2,l} + a_{k,l-2}) with c1 dx, c1 dy
        // formed once per order: one multiply fewer per term
        const T c1 = -(T)(2 * N - 1) * in_, c2 = -(T)(N - 1) * in_;
        const T c1x = c1 * dx, c1y = c1 * dy;
#pragma unroll
        for (int k = 0; k <= N; k++) {
            const int l = N - k;
            T v;
            if (k >= 1 && l >= 1) v = c1x * a[gx_mi(k - 1, l)] + c1y * a[gx_mi(k, l - 1)];
            else if (k >= 1) v = c1x * a[gx_mi(k - 1, l)];
            else v = c1y * a[gx_mi(k, l - 1)];
            if (k >= 2 && l >= 2) v += c2 * (a[gx_mi(k - 2, l)] + a[gx_mi(k, l - 2)]);
            else if (k >= 2) v += c2 * a[gx_mi(k - 2, l)];
            else if (l >= 2) v += c2 * a[gx_mi(k, l - 2)];
            a[gx_mi(k, l)] = v;
            const T Av = (k <= 1 && l <= 1) ? v : v * (T)ff_const(k, l);
            // all splits (k, l) = X + Y with |X| <= p, |Y| <= p
#pragma unroll
            for (int yi = (k > P ? k - P : 0); yi <= (k < P ? k : P); yi++)
#pragma unroll
                for (int yj = (l > P ? l - P : 0); yj <= (l < P ? l : P); yj++) {
                    const int xi = k - yi, xj = l - yj;
                    if (yi + yj <= P && xi + xj <= P) out[gx_mi(xi, xj)] += in[gx_mi(yi, yj)] * Av;
                }
        }
        m2l_order<P, N + 1, T>(dx, dy, ir2, a, in, out);
    }
}

template <int P, class T>
__device__ __forceinline__ void m2l_fused_core(T dx, T dy, T eps2, const T *in, T *out) {
    T r2 = dx * dx + dy * dy + eps2;
    T ir = rsqrt_t<T>(r2);
    T ir2 = ir * ir;
    out[0] += in[0] * ir;
    if constexpr (P <= 8) {
        T a[nc2(2 * P)];
        a[0] = ir;
        m2l_order<P, 1, T>(dx, dy, ir2, a, in, out);
    } else {
        // high orders: run-time loop bounds keep the code size bounded
        const int PP = gx_rt_order(P);
        const int Q = 2 * PP;
        T a[nc2(2 * P)];
        a[0] = ir;
        for (int n = 1; n <= Q; n++) {
            const T in_ = tab_inv<T>(n) * ir2;
            const T c1 = -(T)(2 * n - 1) * in_, c2 = -(T)(n - 1) * in_;
            for (int k = 0; k <= n; k++) {
                const int l = n - k;
                T s1, s2 = T(0);
                if (k >= 1 && l >= 1) s1 = dx * a[gx_mi(k - 1, l)] + dy * a[gx_mi(k, l - 1)];
                else if (k >= 1) s1 = dx * a[gx_mi(k - 1, l)];
                else s1 = dy * a[gx_mi(k, l - 1)];
                if (k >= 2) s2 += a[gx_mi(k - 2, l)];
                if (l >= 2) s2 += a[gx_mi(k, l - 2)];
                const T v = n >= 2 ? c1 * s1 + c2 * s2 : c1 * s1;
                a[gx_mi(k, l)] = v;
                const T Av = n >= 2 ? v * tab_ff<T>(k, l) : v;
                for (int yi = (k > PP ? k - PP : 0); yi <= (k < PP ? k : PP); yi++)
                    for (int yj = (l > PP ? l - PP : 0); yj <= (l < PP ? l : PP); yj++) {
                        const int xi = k - yi, xj = l - yj;
                        if (yi + yj <= PP && xi + xj <= PP) out[gx_mi(xi, xj)] += in[gx_mi(yi, yj)] * Av;
                    }
            }
        }
    }
}

// FP32 at p >= 6: the order-2p derivatives reach R^-(4p+1) (2p)!, beyond the FP32
// range for R ~ 0.1.  The 1/R kernel is homogeneous of degree -1 in (d, eps), so the
// derivatives are formed at unit distance, d' = d/R, and the powers of 1/R go to the
// operands:  out[X] += R^-(1+|X|) sum_Y (in[Y] R^-|Y|) A'[X+Y].
template <int P, class T>
__device__ __forceinline__ void m2l_fused(T dx, T dy, T eps2, const T *in, T *out) {
    if constexpr (sizeof(T) == 4 && P >= 6) {
        constexpr int NC = nc2(P);
        const int PP = gx_rt_order(P);
        const T ir = rsqrt_t<T>(dx * dx + dy * dy + eps2);
        T pw[P + 2];
        pw[0] = T(1);
#pragma unroll
        for (int q = 1; q <= PP + 1; q++) pw[q] = pw[q - 1] * ir;
        T sin_[NC], sout[NC];
#pragma unroll
        for (int yi = 0; yi <= PP; yi++)
#pragma unroll
            for (int yj = 0; yj <= PP - yi; yj++) {
                sin_[gx_mi(yi, yj)] = in[gx_mi(yi, yj)] * pw[yi + yj];
                sout[gx_mi(yi, yj)] = T(0);
            }
        m2l_fused_core<P, T>(dx * ir, dy * ir, eps2 * (ir * ir), sin_, sout);
#pragma unroll
        for (int xi = 0; xi <= PP; xi++)
#pragma unroll
            for (int xj = 0; xj <= PP - xi; xj++) out[gx_mi(xi, xj)] += sout[gx_mi(xi, xj)] * pw[1 + xi + xj];
    } else {
        m2l_fused_core<P, T>(dx, dy, eps2, in, out);
    }
}

// REF mode: derivative sets from the first-inserter table (FP64).
template <int P>
__global__ void __launch_bounds__(128) k_m2l_ref(int64_t nn, const uint32_t *__restrict__ vdata,
                                                 const uint8_t *__restrict__ vlen, const int64_t *__restrict__ voff,
                                                 const int32_t *__restrict__ did, const double *__restrict__ G,
                                                 const double *__restrict__ M, double *__restrict__ L) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<double>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    (void)NCr;
    constexpr int S = 2 * P + 1;
    int64_t node = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (node >= nn) return;
    int len = vlen[node];
    double acc[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) acc[k] = 0.0;
    for (int s = lane; s < len; s += 32) {
        uint32_t src = vdata[node * GX_LIST_CAP + s];
        const double *g = G + (int64_t)did[voff[node] + s] * (S * S);
        double ms[NC];
        load_row<NC>(M + (int64_t)src * NS, ms);
#pragma unroll
        for (int i = 0; i <= PP; i++)
#pragma unroll
            for (int j = 0; j <= PP - i; j++) {
                double mv = ms[gx_mi(i, j)];
                if (mv == 0.0) continue;  // lib.rs:1252: zero source terms are skipped
                double sm = ((i + j) & 1) ? -mv : mv;
#pragma unroll
                for (int oi = 0; oi <= PP; oi++)
#pragma unroll
                    for (int oj = 0; oj <= PP - oi; oj++)
                        acc[gx_mi(oi, oj)] += sm * g[gx_kdi(i + oi, j + oj, P)];
            }
    }
#pragma unroll
    for (int oi = 0; oi <= PP; oi++)
#pragma unroll
        for (int oj = 0; oj <= PP - oi; oj++) {
            int k = gx_mi(oi, oj);
            double v = warp_sum_t<double>(acc[k]);
            if (lane == (k & 31)) L[node * NS + k] = v * tab_ifp<double>(oi, oj);
        }
}

// EXACT / ACCURATE M2L of one target over its sources idx[st .. st + len): lane l takes
// sources l, l + 32, ...; acc holds the lane's unscaled sum over M'[S] A[S+T].
template <int P, class T, class IDX>
__device__ __forceinline__ void m2l_sources(const IDX *__restrict__ idx, int64_t st, int len, int lane, double tcx,
                                            double tcy, float4 thl, const double *__restrict__ comx,
                                            const double *__restrict__ comy, const float4 *__restrict__ comhl, T eps2,
                                            const T *__restrict__ M, T *acc) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    // the next source index is fetched one iteration ahead, and the source row is
    // requested before the derivatives are formed, so both latencies overlap compute
    int64_t src = lane < len ? (int64_t)idx[st + lane] : 0;
    for (int s = lane; s < len; s += 32) {
        int64_t nsrc = s + 32 < len ? (int64_t)idx[st + s + 32] : 0;
        T ms[NC];
        load_row<NC>(M + src * NS, ms);
        T dx, dy;
        if constexpr (sizeof(T) == 4) {
            // COMs as FP32 (hi, lo) pairs: the offset is exact to FP32 rounding without
            // FP64 work (a compile-time choice: a run-time branch would be if-converted
            // and issue the FP64 path's instructions, predicated off, on every pair)
            float4 shl = comhl[src];
            dx = (T)((thl.x - shl.x) + (thl.y - shl.y));
            dy = (T)((thl.z - shl.z) + (thl.w - shl.w));
        } else {
            dx = (T)(tcx - comx[src]);
            dy = (T)(tcy - comy[src]);
        }
#pragma unroll
        for (int i = 0; i <= PP; i++)
#pragma unroll
            for (int j = 0; j <= PP - i; j++)
                if ((i + j) & 1) ms[gx_mi(i, j)] = -ms[gx_mi(i, j)];
        m2l_fused<P, T>(dx, dy, eps2, ms, acc);
        src = nsrc;
    }
}

// EXACT / ACCURATE: per-pair derivatives.  Lists given as start/count per node.
template <int P, class T, class IDX>
// FP32 at p <= 4 fits 64 registers without spills: 8 blocks (32 warps) per SM
__global__ void __launch_bounds__(128, (sizeof(T) == 4 && P <= 4) ? 8 : 1) k_m2l_exact(int64_t nn, const IDX *__restrict__ idx,
                                                   const int64_t *__restrict__ start, const int32_t *__restrict__ cnt,
                                                   const uint8_t *__restrict__ cnt8, int64_t fixed_stride,
                                                   const double *__restrict__ comx, const double *__restrict__ comy,
                                                   const float4 *__restrict__ comhl, double eps2d,
                                                   const T *__restrict__ M, T *__restrict__ L) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    (void)NCr;
    int64_t node = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (node >= nn) return;
    int64_t st = start ? start[node] : node * fixed_stride;
    int len = cnt ? cnt[node] : (int)cnt8[node];
    float4 thl = make_float4(0.f, 0.f, 0.f, 0.f);
    if constexpr (sizeof(T) == 4) thl = comhl[node];
    T acc[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) acc[k] = T(0);
    m2l_sources<P, T, IDX>(idx, st, len, lane, comx[node], comy[node], thl, comx, comy, comhl, (T)eps2d, M, acc);
    // G = -A: L[T] = -(1/T!) sum_S M'[S] A[S+T]
#pragma unroll
    for (int oi = 0; oi <= PP; oi++)
#pragma unroll
        for (int oj = 0; oj <= PP - oi; oj++) {
            int k = gx_mi(oi, oj);
            T v = warp_sum_t<T>(acc[k]);
            if (lane == (k & 31)) L[node * NS + k] = v * -tab_ifp<T>(oi, oj);
        }
}

// ACCURATE M2L over work units: every far list is cut into units of at most
// GX_M2L_UNIT sources (one warp each), so a node near the centre of a wide halo, with
// tens of thousands of far sources, is spread over many warps instead of running as
// one straggler.  A node with one unit writes its local directly; otherwise each unit
// writes its warp-reduced partial and k_m2l_combine sums them in unit order.
template <int P, class T>
__global__ void __launch_bounds__(128, (sizeof(T) == 4 && P <= 4) ? 8 : 1) k_m2l_units(
    int64_t n_units, const int32_t *__restrict__ unode, const int64_t *__restrict__ ustart,
    const int32_t *__restrict__ ulen, const int64_t *__restrict__ node_u, const int32_t *__restrict__ idx,
    const double *__restrict__ comx, const double *__restrict__ comy, const float4 *__restrict__ comhl, double eps2d,
    const T *__restrict__ M, T *__restrict__ L, T *__restrict__ part) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    (void)NCr;
    int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (u >= n_units) return;
    const int64_t node = unode[u];
    const bool single = node_u[node + 1] - node_u[node] == 1;
    float4 thl = make_float4(0.f, 0.f, 0.f, 0.f);
    if constexpr (sizeof(T) == 4) thl = comhl[node];
    T acc[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) acc[k] = T(0);
    m2l_sources<P, T, int32_t>(idx, ustart[u], ulen[u], lane, comx[node], comy[node], thl, comx, comy, comhl,
                               (T)eps2d, M, acc);
#pragma unroll
    for (int oi = 0; oi <= PP; oi++)
#pragma unroll
        for (int oj = 0; oj <= PP - oi; oj++) {
            int k = gx_mi(oi, oj);
            T v = warp_sum_t<T>(acc[k]);
            if (lane == (k & 31)) {
                if (single) L[node * NS + k] = v * -tab_ifp<T>(oi, oj);
                else part[u * NS + k] = v;
            }
        }
}

// Nodes cut into several M2L units: the local is the sum of the units' partials in
// unit order.  One thread per (node, coefficient).
template <int P, class T>
__global__ void k_m2l_combine(int64_t nn, const int64_t *__restrict__ node_u, const T *__restrict__ part,
                              T *__restrict__ L) {
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
    int n = 0;  // coefficient k = gx_mi(oi, oj): n(n+1)/2 + oj with n = oi + oj
    while ((n + 1) * (n + 2) / 2 <= k) n++;
    const int oj = k - n * (n + 1) / 2, oi = n - oj;
    L[node * NS + k] = s * -tab_ifp<T>(oi, oj);
}

// ---------------------------------------------------------------- L2L
// L_c[I,J] += sum_{i>=I, j>=J} L_P[i,j] C(i,I) C(j,J) dx^(i-I) dy^(j-J), one thread per child.
template <int P, class T>
__device__ __forceinline__ void l2l_shift(const T *__restrict__ LP, T dx, T dy, T *out) {
    const int PP = gx_rt_order(P);
    T px[P + 1], py[P + 1];
    px[0] = T(1);
    py[0] = T(1);
#pragma unroll
    for (int q = 1; q <= PP; q++) {
        px[q] = px[q - 1] * dx;
        py[q] = py[q - 1] * dy;
    }
    T lp[nc2(P)];
    load_row<nc2(P)>(LP, lp);
#pragma unroll
    for (int oi = 0; oi <= PP; oi++)
#pragma unroll
        for (int oj = 0; oj <= PP - oi; oj++) {
            T sum = T(0);
#pragma unroll
            for (int i = oi; i <= PP; i++)
#pragma unroll
                for (int j = oj; j <= PP - i; j++)
                    sum += lp[gx_mi(i, j)] * (tab_binom<T>(i, oi) * tab_binom<T>(j, oj)) * px[i - oi] * py[j - oj];
            out[gx_mi(oi, oj)] += sum;
        }
}

// Top-down modes: only the leaves' locals are consumed (by L2P), and translating a
// local expansion is exact for polynomials, so shifting every ancestor's M2L local
// straight to the leaf equals the level-by-level L2L chain.  One warp per leaf, one
// lane per ancestor (from the ancestor table anc[level * nl + leaf]), then a warp
// reduction: a single launch instead of one per level.  Ancestors without far
// interactions (has_far = 0) hold a zero local and are skipped.
template <int P, class T>
__global__ void __launch_bounds__(128) k_l2l_direct(int64_t nl, int n_levels, const int32_t *__restrict__ anc,
                                                    const uint8_t *__restrict__ has_far, const double *__restrict__ comx,
                                                    const double *__restrict__ comy, const T *__restrict__ L,
                                                    T *__restrict__ Lout) {
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
        if (a == (int32_t)leaf) {
            T own[NC];
            load_row<NC>(L + leaf * NS, own);
#pragma unroll
            for (int k = 0; k < NCr; k++) out[k] += own[k];
        } else {
            l2l_shift<P, T>(L + (int64_t)a * NS, (T)(comx[leaf] - comx[a]), (T)(comy[leaf] - comy[a]), out);
        }
    }
#pragma unroll
    for (int k = 0; k < NCr; k++) {
        T v = warp_sum_t<T>(out[k]);
        if (lane == (k & 31)) Lout[leaf * NS + k] = v;
    }
}

// REF: Lout[leaf] = L[leaf] + shift(L[parent(leaf)])
template <int P, class T>
__global__ void __launch_bounds__(128) k_l2l_ref_leaves(int64_t nl, const int32_t *__restrict__ parent,
                                                        const double *__restrict__ comx, const double *__restrict__ comy,
                                                        const T *__restrict__ L, T *__restrict__ Lout) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    int64_t leaf = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= nl) return;
    int32_t par = parent[leaf];
    T out[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) out[k] = L[leaf * NS + k];
    if (par >= 0)
        l2l_shift<P, T>(L + (int64_t)par * NS, (T)(comx[leaf] - comx[par]), (T)(comy[leaf] - comy[par]), out);
#pragma unroll
    for (int k = 0; k < NCr; k++) Lout[leaf * NS + k] = out[k];
}

// ---------------------------------------------------------------- L2P + P2P
// One warp per target leaf, one lane per target body (chunks of 32 for larger
// leaves).  The source-leaf list is read 32 entries at a time (one coalesced load)
// and broadcast by shuffles; each source leaf (<= 32 bodies) is loaded one body per
// lane, staged in shared memory and read back as a broadcast, and the next leaf's
// load is issued before the current leaf is computed, so its latency is hidden.
// The target leaf itself is handled in a separate branch (i == j is skipped there),
// keeping the common loop free of the self test.

// L2P (lib.rs:1321-1345) for one body at (du, dv) from the leaf COM
template <int P, class T>
__device__ __forceinline__ void l2p_eval(const T *__restrict__ Ll, T du, T dv, T &fx, T &fy) {
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    (void)NCr;
    T px[P + 1], py[P + 1];
    px[0] = T(1);
    py[0] = T(1);
#pragma unroll
    for (int q = 1; q <= PP; q++) {
        px[q] = px[q - 1] * du;
        py[q] = py[q - 1] * dv;
    }
    fx = T(0);
    fy = T(0);
#pragma unroll
    for (int a = 0; a <= PP; a++)
#pragma unroll
        for (int b = 0; b <= PP - a; b++) {
            T c = Ll[gx_mi(a, b)];
            if (a >= 1) fx += c * (T)a * px[a - 1] * py[b];
            if (b >= 1) fy += c * (T)b * px[a] * py[b - 1];
        }
}

// Work items: the source list of every target leaf is cut into items of at most
// P2P_K source leaves; one warp per item writes per-body partial accelerations to
// its own slot, so the work per warp is bounded however uneven the lists are
// (Plummer core leaves have hundreds of near leaves, halo leaves a few).  A second
// kernel evaluates L2P and adds the partials of each leaf in item order, so the
// result does not depend on scheduling.

// FP64 partials: sum_j m_j (x_j - x_i) / (r^2+eps^2)^(3/2)
__global__ void __launch_bounds__(128) k_p2p64_items(int64_t n_items, const int32_t *__restrict__ item_leaf,
                                                     const int64_t *__restrict__ item_qb, const int32_t *__restrict__ item_nq,
                                                     const double *__restrict__ x, const double *__restrict__ y,
                                                     const double *__restrict__ m, const int32_t *__restrict__ bs,
                                                     const int32_t *__restrict__ be, const int32_t *__restrict__ src_idx,
                                                     const uint32_t *__restrict__ p2p_mask, double eps2, int tchunks,
                                                     double2 *__restrict__ part) {
    __shared__ double3 sb[4][32];
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t it = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (it >= n_items) return;
    int32_t leaf = item_leaf[it];
    int64_t qb = item_qb[it];
    int nq = item_nq[it];
    if (nq < 0) return;  // an M2P item of the near-list split (k_m2p)
    int32_t t0 = bs[leaf], t1 = be[leaf];
    int sl = lane < nq ? src_idx[qb + lane] : -1;
    int sbeg = sl >= 0 ? bs[sl] : 0, send = sl >= 0 ? be[sl] : 0;
    // the body-level P2L (p2p_mask != null): a row's masked bodies are skipped here
    const uint32_t skip = (p2p_mask && sl >= 0) ? p2p_mask[qb + lane] : 0u;
    auto fetch = [&](int k, int sc) -> double3 {
        int s0 = __shfl_sync(0xffffffffu, sbeg, k) + sc, s1 = __shfl_sync(0xffffffffu, send, k);
        int j = s0 + lane;
        return (j < s1) ? make_double3(x[j], y[j], m[j]) : make_double3(0.0, 0.0, 0.0);
    };
    for (int tc = 0; tc < tchunks; tc++) {
        int32_t i = t0 + tc * 32 + lane;
        bool valid = i < t1;
        double xi = valid ? x[i] : 0.0, yi = valid ? y[i] : 0.0;
        double accx = 0.0, accy = 0.0;
        if (t0 + tc * 32 < t1) {
            double3 cur = fetch(0, 0);
            for (int k = 0; k < nq; k++) {
                int s0 = __shfl_sync(0xffffffffu, sbeg, k), s1 = __shfl_sync(0xffffffffu, send, k);
                int srcl = __shfl_sync(0xffffffffu, sl, k);
                const uint32_t sk = __shfl_sync(0xffffffffu, skip, k);
                for (int sc = 0; sc < s1 - s0; sc += 32) {
                    double3 nxt;
                    if (sc + 32 < s1 - s0) nxt = fetch(k, sc + 32);
                    else nxt = (k + 1 < nq) ? fetch(k + 1, 0) : make_double3(0.0, 0.0, 0.0);
                    __syncwarp();
                    sb[w][lane] = cur;
                    __syncwarp();
                    int ns = min(32, s1 - s0 - sc);
                    if (srcl == leaf) {
                        for (int kk = 0; kk < ns; kk++) {
                            double3 bb = sb[w][kk];
                            double dx = bb.x - xi, dy = bb.y - yi;
                            double ir = rsqrt(dx * dx + dy * dy + eps2);
                            double f = bb.z * (ir * ir * ir);
                            if (s0 + sc + kk == i) f = 0.0;
                            accx += f * dx;
                            accy += f * dy;
                        }
                    } else if (sk) {
                        for (int kk = 0; kk < ns; kk++) {
                            if ((sk >> kk) & 1u) continue;  // leaves of at most 32 bodies: sc = 0
                            double3 bb = sb[w][kk];
                            double dx = bb.x - xi, dy = bb.y - yi;
                            double ir = rsqrt(dx * dx + dy * dy + eps2);
                            double f = bb.z * (ir * ir * ir);
                            accx += f * dx;
                            accy += f * dy;
                        }
                    } else {
#pragma unroll 4
                        for (int kk = 0; kk < ns; kk++) {
                            double3 bb = sb[w][kk];
                            double dx = bb.x - xi, dy = bb.y - yi;
                            double ir = rsqrt(dx * dx + dy * dy + eps2);
                            double f = bb.z * (ir * ir * ir);
                            accx += f * dx;
                            accy += f * dy;
                        }
                    }
                    cur = nxt;
                }
            }
        }
        part[(it * tchunks + tc) * 32 + lane] = make_double2(accx, accy);
    }
}

// FP32 partials on coordinates relative to the target leaf's COM.  Bodies come packed
// as (x - com_leaf, y - com_leaf, m) in FP32 (written by P2M); a source leaf is moved
// into the target's frame by one FP32 shift per leaf pair, formed in FP64 and rounded once.
// 7 blocks per SM: 72 registers, no spills (left alone, ptxas picks 64 and spills)
__global__ void __launch_bounds__(128, 7) k_p2p32_items(int64_t n_items, const int32_t *__restrict__ item_leaf,
                                                     const int64_t *__restrict__ item_qb, const int32_t *__restrict__ item_nq,
                                                     const float4 *__restrict__ pos, const double *__restrict__ comx,
                                                     const double *__restrict__ comy, const int32_t *__restrict__ bs,
                                                     const int32_t *__restrict__ be, const int32_t *__restrict__ src_idx,
                                                     float eps2, int tchunks, float2 *__restrict__ part) {
    // staged sources, one row of 32 per warp, as x / y / m planes so that one
    // broadcast 16-byte load yields the x (or y, m) of four consecutive sources
    __shared__ __align__(16) float sx[4][32], sy[4][32], sm[4][32];
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // one warp per item (a grid-stride loop, launched with one warp for every item)
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t it = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < n_items; it += nwarps) {
        int32_t leaf = item_leaf[it];
        int64_t qb = item_qb[it];
        int nq = item_nq[it];
        if (nq < 0) continue;  // an M2P item of the near-list split (k_m2p)
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
        auto fetch = [&](int k, int sc) -> float4 {
            int s0 = __shfl_sync(0xffffffffu, sbeg, k) + sc, s1 = __shfl_sync(0xffffffffu, send, k);
            float gx = __shfl_sync(0xffffffffu, shx, k), gy = __shfl_sync(0xffffffffu, shy, k);
            int j = s0 + lane;
            float4 v = (j < s1) ? pos[j] : make_float4(0.f, 0.f, 0.f, 0.f);
            v.x += gx;
            v.y += gy;
            return v;
        };
        for (int tc = 0; tc < tchunks; tc++) {
            int32_t i = t0 + tc * 32 + lane;
            bool valid = i < t1;
            float4 me = valid ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
            float xi = me.x, yi = me.y;
            const uint64_t XI = pk2(xi, xi), YI = pk2(yi, yi), E2 = pk2(eps2, eps2);
            // full 32-source rows: four packed accumulator chains (sources 4q, 4q+1 in
            // AXa/AYa; 4q+2, 4q+3 in AXb/AYb) so consecutive updates are independent;
            // the own leaf and partial rows go through the scalar loop into axs/ays
            uint64_t AXa = 0, AYa = 0, AXb = 0, AYb = 0;  // bit pattern 0 = (0.f, 0.f)
            float axs = 0.f, ays = 0.f;
            if (t0 + tc * 32 < t1) {
                float4 cur = fetch(0, 0);
                for (int k = 0; k < nq; k++) {
                    int s0 = __shfl_sync(0xffffffffu, sbeg, k), s1 = __shfl_sync(0xffffffffu, send, k);
                    int srcl = __shfl_sync(0xffffffffu, sl, k);
                    for (int sc = 0; sc < s1 - s0; sc += 32) {
                        float4 nxt;
                        if (sc + 32 < s1 - s0) nxt = fetch(k, sc + 32);
                        else nxt = (k + 1 < nq) ? fetch(k + 1, 0) : make_float4(0.f, 0.f, 0.f, 0.f);
                        __syncwarp();
                        sx[w][lane] = cur.x;
                        sy[w][lane] = cur.y;
                        sm[w][lane] = cur.z;
                        __syncwarp();
                        int ns = min(32, s1 - s0 - sc);
                        // four sources kk .. kk+3 on packed FP32
                        auto quad = [&](int kk) {
                            float4 X = *reinterpret_cast<const float4 *>(&sx[w][kk]);
                            float4 Y = *reinterpret_cast<const float4 *>(&sy[w][kk]);
                            float4 Mq = *reinterpret_cast<const float4 *>(&sm[w][kk]);
                            uint64_t dx0 = sub2(pk2(X.x, X.y), XI), dy0 = sub2(pk2(Y.x, Y.y), YI);
                            uint64_t dx1 = sub2(pk2(X.z, X.w), XI), dy1 = sub2(pk2(Y.z, Y.w), YI);
                            uint64_t r0 = fma2(dx0, dx0, fma2(dy0, dy0, E2));
                            uint64_t r1 = fma2(dx1, dx1, fma2(dy1, dy1, E2));
                            float ra, rb;
                            upk2(r0, ra, rb);
                            uint64_t i0 = pk2(rsqrt_fast(ra), rsqrt_fast(rb));
                            upk2(r1, ra, rb);
                            uint64_t i1 = pk2(rsqrt_fast(ra), rsqrt_fast(rb));
                            uint64_t f0 = mul2(pk2(Mq.x, Mq.y), mul2(mul2(i0, i0), i0));
                            uint64_t f1 = mul2(pk2(Mq.z, Mq.w), mul2(mul2(i1, i1), i1));
                            AXa = fma2(f0, dx0, AXa);
                            AYa = fma2(f0, dy0, AYa);
                            AXb = fma2(f1, dx1, AXb);
                            AYb = fma2(f1, dy1, AYb);
                        };
                        const bool own = srcl == leaf;
                        int k0 = 0;  // sources below k0 are done
                        if (!own) {
                            if (ns == 32) {
#pragma unroll
                                for (int kk = 0; kk < 32; kk += 4) quad(kk);
                                k0 = 32;
                            } else {
                                // partial rows (leaves below n_max, or n_max = 16): packed quads, scalar tail
                                for (k0 = 0; k0 + 4 <= ns; k0 += 4) quad(k0);
                            }
                        }
                        for (int kk = k0; kk < ns; kk++) {
                            float dx = sx[w][kk] - xi, dy = sy[w][kk] - yi;
                            float ir = rsqrt_fast(fmaf(dx, dx, fmaf(dy, dy, eps2)));
                            float fk = sm[w][kk] * (ir * ir * ir);
                            fk = (own && s0 + sc + kk == i) ? 0.f : fk;
                            axs = fmaf(fk, dx, axs);
                            ays = fmaf(fk, dy, ays);
                        }
                        cur = nxt;
                    }
                }
            }
            float a0, a1, a2, a3, b0, b1, b2, b3;
            upk2(AXa, a0, a1);
            upk2(AXb, a2, a3);
            upk2(AYa, b0, b1);
            upk2(AYb, b2, b3);
            part[(it * tchunks + tc) * 32 + lane] =
                make_float2(((a0 + a1) + (a2 + a3)) + axs, ((b0 + b1) + (b2 + b3)) + ays);
        }
    }
}

// The one-row kernel with one target per lane and every source of the row, for leaves
// of at most 16 bodies (n_max <= 16), where the second target of k_p2p32_rows would be
// empty and a row holds only half a warp of sources: partial rows run their whole
// quads packed and the rest scalar.
__global__ void __launch_bounds__(128, 8) k_p2p32_rows1(int64_t n_items, const int32_t *__restrict__ item_leaf,
                                                    const int64_t *__restrict__ item_qb, const int32_t *__restrict__ item_nq,
                                                    const float4 *__restrict__ pos, const double *__restrict__ comx,
                                                    const double *__restrict__ comy, const int32_t *__restrict__ bs,
                                                    const int32_t *__restrict__ be, const int32_t *__restrict__ src_idx,
                                                    float eps2, float2 *__restrict__ part) {
    __shared__ __align__(16) float sx[4][32], sy[4][32], sm[4][32];
    __shared__ __align__(16) int4 meta[4][32];  // per source leaf: begin, end, shift x, shift y (FP32 bits)
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t it = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < n_items; it += nwarps) {
        const int32_t leaf = item_leaf[it];
        const int nq = item_nq[it];
        if (nq < 0) continue;  // an M2P item of the near-list split (k_m2p)
        const int32_t t0 = bs[leaf], t1 = be[leaf];
        bool own_lane = false;
        __syncwarp();  // the previous item's reads of meta[w] are done
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
        const float4 me = i < t1 ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        const uint64_t XI = pk2(me.x, me.x), YI = pk2(me.y, me.y), E2 = pk2(eps2, eps2);
        uint64_t AXa = 0, AYa = 0, AXb = 0, AYb = 0;  // bit pattern 0 = (0.f, 0.f)
        float axs = 0.f, ays = 0.f;
        auto fetch = [&](int4 m) -> float4 {
            int j = m.x + lane;
            float4 v = j < m.y ? pos[j] : make_float4(0.f, 0.f, 0.f, 0.f);
            v.x += __int_as_float(m.z);
            v.y += __int_as_float(m.w);
            return v;
        };
        float4 cur = nq > 0 ? fetch(meta[w][0]) : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int k = 0; k < nq; k++) {
            const float4 nxt = k + 1 < nq ? fetch(meta[w][k + 1]) : make_float4(0.f, 0.f, 0.f, 0.f);
            __syncwarp();
            sx[w][lane] = cur.x;
            sy[w][lane] = cur.y;
            sm[w][lane] = cur.z;
            __syncwarp();
            const int2 se = *reinterpret_cast<const int2 *>(&meta[w][k]);  // this row's begin, end
            const int ns = se.y - se.x;
            auto quad = [&](int kk) {
                float4 X = *reinterpret_cast<const float4 *>(&sx[w][kk]);
                float4 Y = *reinterpret_cast<const float4 *>(&sy[w][kk]);
                float4 Mq = *reinterpret_cast<const float4 *>(&sm[w][kk]);
                uint64_t dx0 = sub2(pk2(X.x, X.y), XI), dy0 = sub2(pk2(Y.x, Y.y), YI);
                uint64_t dx1 = sub2(pk2(X.z, X.w), XI), dy1 = sub2(pk2(Y.z, Y.w), YI);
                uint64_t r0 = fma2(dx0, dx0, fma2(dy0, dy0, E2));
                uint64_t r1 = fma2(dx1, dx1, fma2(dy1, dy1, E2));
                float ra, rb;
                upk2(r0, ra, rb);
                uint64_t i0 = pk2(rsqrt_fast(ra), rsqrt_fast(rb));
                upk2(r1, ra, rb);
                uint64_t i1 = pk2(rsqrt_fast(ra), rsqrt_fast(rb));
                uint64_t f0 = mul2(pk2(Mq.x, Mq.y), mul2(mul2(i0, i0), i0));
                uint64_t f1 = mul2(pk2(Mq.z, Mq.w), mul2(mul2(i1, i1), i1));
                AXa = fma2(f0, dx0, AXa);
                AYa = fma2(f0, dy0, AYa);
                AXb = fma2(f1, dx1, AXb);
                AYb = fma2(f1, dy1, AYb);
            };
            int k0 = 0;  // sources below k0 are done
            if (k != kown) {
                if (ns == 32) {
#pragma unroll
                    for (int kk = 0; kk < 32; kk += 4) quad(kk);
                    k0 = 32;
                } else {
                    for (k0 = 0; k0 + 4 <= ns; k0 += 4) quad(k0);
                }
            }
            for (int kk = k0; kk < ns; kk++) {
                float xi, yi, dum;
                upk2(XI, xi, dum);
                upk2(YI, yi, dum);
                float dx = sx[w][kk] - xi, dy = sy[w][kk] - yi;
                float ir = rsqrt_fast(fmaf(dx, dx, fmaf(dy, dy, eps2)));
                float fk = sm[w][kk] * (ir * ir * ir);
                fk = (k == kown && se.x + kk == i) ? 0.f : fk;
                axs = fmaf(fk, dx, axs);
                ays = fmaf(fk, dy, ays);
            }
            cur = nxt;
        }
        float a0, a1, a2, a3, b0, b1, b2, b3;
        upk2(AXa, a0, a1);
        upk2(AXb, a2, a3);
        upk2(AYa, b0, b1);
        upk2(AYb, b2, b3);
        part[it * 32 + lane] = make_float2(((a0 + a1) + (a2 + a3)) + axs, ((b0 + b1) + (b2 + b3)) + ays);
    }
}

// The same near field when every leaf holds at most 32 bodies (n_max <= 32): each
// source leaf is one row, so the item's source-leaf table (first body, end, FP32
// frame shift) is written to shared memory once per item and read back by broadcast
// as the rows go, and there is no row loop.  Each lane takes two targets (t and t + 16)
// and half of every row's sources (the quads 4h, 4h + 8, ... of half h), so one
// broadcast load of four sources serves eight interactions; the two halves' sums of a
// target are added (half 0 first) at the end of the item.  Same per-interaction
// arithmetic as k_p2p32_items.
__global__ void __launch_bounds__(128, 8) k_p2p32_rows(int64_t n_items, const int32_t *__restrict__ item_leaf,
                                                    const int64_t *__restrict__ item_qb, const int32_t *__restrict__ item_nq,
                                                    const float4 *__restrict__ pos, const double *__restrict__ comx,
                                                    const double *__restrict__ comy, const int32_t *__restrict__ bs,
                                                    const int32_t *__restrict__ be, const int32_t *__restrict__ src_idx,
                                                    float eps2, float2 *__restrict__ part) {
    __shared__ __align__(16) float sx[4][32], sy[4][32], sm[4][32];
    __shared__ __align__(16) int4 meta[4][32];  // per source leaf: begin, end, shift x, shift y (FP32 bits)
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int half = lane >> 4, tl = lane & 15;  // lane: targets tl and tl + 16, source quads of its half
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t it = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < n_items; it += nwarps) {
        const int32_t leaf = item_leaf[it];
        const int nq = item_nq[it];
        if (nq < 0) continue;  // an M2P item of the near-list split (k_m2p)
        const int32_t t0 = bs[leaf], t1 = be[leaf];
        bool own_lane = false;
        __syncwarp();  // the previous item's reads of meta[w] are done
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
        const int32_t iA = t0 + tl, iB = t0 + tl + 16;
        const float4 mA = iA < t1 ? pos[iA] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 mB = iB < t1 ? pos[iB] : make_float4(0.f, 0.f, 0.f, 0.f);
        const uint64_t XA = pk2(mA.x, mA.x), YA = pk2(mA.y, mA.y), XB = pk2(mB.x, mB.x), YB = pk2(mB.y, mB.y);
        const uint64_t E2 = pk2(eps2, eps2);
        uint64_t AXA = 0, AYA = 0, AXB = 0, AYB = 0;
        float sxA = 0.f, syA = 0.f, sxB = 0.f, syB = 0.f;
        auto fetch = [&](int4 m) -> float4 {
            int j = m.x + lane;
            float4 v = j < m.y ? pos[j] : make_float4(0.f, 0.f, 0.f, 0.f);
            v.x += __int_as_float(m.z);
            v.y += __int_as_float(m.w);
            return v;
        };
        float4 cur = nq > 0 ? fetch(meta[w][0]) : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int k = 0; k < nq; k++) {
            const float4 nxt = k + 1 < nq ? fetch(meta[w][k + 1]) : make_float4(0.f, 0.f, 0.f, 0.f);
            __syncwarp();
            sx[w][lane] = cur.x;
            sy[w][lane] = cur.y;
            sm[w][lane] = cur.z;
            __syncwarp();
            const int2 se = *reinterpret_cast<const int2 *>(&meta[w][k]);  // this row's begin, end
            const int ns = se.y - se.x;
            if (ns == 32 && k != kown) {
                // full rows of other leaves on packed .f32x2: sources (2v, 2v + 1) per instruction
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int kk = 8 * q + 4 * half;
                    float4 X = *reinterpret_cast<const float4 *>(&sx[w][kk]);
                    float4 Y = *reinterpret_cast<const float4 *>(&sy[w][kk]);
                    float4 Mq = *reinterpret_cast<const float4 *>(&sm[w][kk]);
                    const uint64_t X0 = pk2(X.x, X.y), X1 = pk2(X.z, X.w), Y0 = pk2(Y.x, Y.y), Y1 = pk2(Y.z, Y.w);
                    const uint64_t M0 = pk2(Mq.x, Mq.y), M1 = pk2(Mq.z, Mq.w);
                    auto pair = [&](uint64_t XS, uint64_t YS, uint64_t MS, uint64_t XI, uint64_t YI, uint64_t &AX,
                                    uint64_t &AY) {
                        uint64_t dx = sub2(XS, XI), dy = sub2(YS, YI);
                        uint64_t r = fma2(dx, dx, fma2(dy, dy, E2));
                        float ra, rb;
                        upk2(r, ra, rb);
                        uint64_t ir = pk2(rsqrt_fast(ra), rsqrt_fast(rb));
                        uint64_t fq = mul2(MS, mul2(mul2(ir, ir), ir));
                        AX = fma2(fq, dx, AX);
                        AY = fma2(fq, dy, AY);
                    };
                    pair(X0, Y0, M0, XA, YA, AXA, AYA);
                    pair(X0, Y0, M0, XB, YB, AXB, AYB);
                    pair(X1, Y1, M1, XA, YA, AXA, AYA);
                    pair(X1, Y1, M1, XB, YB, AXB, AYB);
                }
            } else {
                // partial or own rows: scalar, each half its own quads
                float xa, ya, xb, yb, d;
                upk2(XA, xa, d);
                upk2(YA, ya, d);
                upk2(XB, xb, d);
                upk2(YB, yb, d);
                for (int q = 0; q < 4; q++)
                    for (int u = 0; u < 4; u++) {
                        const int kk = 8 * q + 4 * half + u;
                        if (kk >= ns) continue;
                        const float xj = sx[w][kk], yj = sy[w][kk], mj = sm[w][kk];
                        float dx = xj - xa, dy = yj - ya;
                        float ir = rsqrt_fast(fmaf(dx, dx, fmaf(dy, dy, eps2)));
                        float fk = mj * (ir * ir * ir);
                        fk = (k == kown && se.x + kk == iA) ? 0.f : fk;
                        sxA = fmaf(fk, dx, sxA);
                        syA = fmaf(fk, dy, syA);
                        dx = xj - xb;
                        dy = yj - yb;
                        ir = rsqrt_fast(fmaf(dx, dx, fmaf(dy, dy, eps2)));
                        fk = mj * (ir * ir * ir);
                        fk = (k == kown && se.x + kk == iB) ? 0.f : fk;
                        sxB = fmaf(fk, dx, sxB);
                        syB = fmaf(fk, dy, syB);
                    }
            }
            cur = nxt;
        }
        float a0, a1, b0, b1, c0, c1, e0, e1;
        upk2(AXA, a0, a1);
        upk2(AYA, b0, b1);
        upk2(AXB, c0, c1);
        upk2(AYB, e0, e1);
        float xA = (a0 + a1) + sxA, yA = (b0 + b1) + syA, xB = (c0 + c1) + sxB, yB = (e0 + e1) + syB;
        // the two halves hold the same targets over different sources: half 0 + half 1
        const float oxA = __shfl_xor_sync(0xffffffffu, xA, 16), oyA = __shfl_xor_sync(0xffffffffu, yA, 16);
        const float oxB = __shfl_xor_sync(0xffffffffu, xB, 16), oyB = __shfl_xor_sync(0xffffffffu, yB, 16);
        float2 res;
        if (half == 0) res = make_float2(xA + oxA, yA + oyA);  // target tl
        else res = make_float2(oxB + xB, oyB + yB);             // target tl + 16 (half 0's part first)
        part[it * 32 + lane] = res;
    }
}

// The near field of k_p2p32_rows with the body-level P2L (leaves of at most 32 bodies):
// row k of an item keeps the bodies of its source leaf outside the plan's mask (the
// masked ones went to the target leaf's local expansion).  The rows' kept bodies are laid
// out as one stream per item in shared memory (entry (row << 5) | body, in row and body
// order) and computed 32 at a time with the packed quads of k_p2p32_rows, the last chunk
// padded with zero-mass sources far away (r^-3 underflows to 0).  The self row is in the
// stream when eps > 0 (each body's term on itself is exactly 0); with eps = 0 it runs
// first, as the scalar own row of k_p2p32_rows.  With empty masks the stream is every body
// of every row, so the same kernel serves the plain split.
__global__ void __launch_bounds__(128, 8) k_p2p32_stream(
    int64_t n_items, const int32_t *__restrict__ item_leaf, const int64_t *__restrict__ item_qb,
    const int32_t *__restrict__ item_nq, const float4 *__restrict__ pos, const double *__restrict__ comx,
    const double *__restrict__ comy, const int32_t *__restrict__ bs, const int32_t *__restrict__ be,
    const int32_t *__restrict__ src_idx, const uint32_t *__restrict__ p2p_mask, float eps2,
    float2 *__restrict__ part) {
    __shared__ __align__(16) float sx[4][32], sy[4][32], sm[4][32];
    __shared__ __align__(16) int4 meta[4][32];  // per source leaf: begin, end, shift x, shift y (FP32 bits)
    __shared__ uint16_t strm[4][32 * 32];       // the item's kept bodies: (row << 5) | body
    const unsigned full = 0xffffffffu;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int half = lane >> 4, tl = lane & 15;  // lane: targets tl and tl + 16, source quads of its half
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const float4 far4 = make_float4(1e18f, 1e18f, 0.f, 0.f);
    const bool self_in_stream = eps2 > 0.f;
    for (int64_t it = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < n_items; it += nwarps) {
        const int32_t leaf = item_leaf[it];
        const int nq = item_nq[it];
        if (nq < 0) continue;  // an M2P item of the near-list split (k_m2p)
        const int32_t t0 = bs[leaf], t1 = be[leaf];
        bool own_lane = false;
        uint32_t keep = 0;
        __syncwarp();  // the previous item's reads of meta[w] and strm[w] are done
        if (lane < nq) {
            const int64_t q = item_qb[it] + lane;
            const int32_t sl = src_idx[q];
            const int32_t b0 = bs[sl], b1 = be[sl];
            const double tcx = comx[leaf], tcy = comy[leaf];
            meta[w][lane] = make_int4(b0, b1, __float_as_int((float)(comx[sl] - tcx)),
                                      __float_as_int((float)(comy[sl] - tcy)));
            own_lane = sl == leaf;
            const int ns = b1 - b0;
            const uint32_t all = ns >= 32 ? full : ((1u << ns) - 1u);
            // with eps > 0 the self row joins the stream: a body against itself has
            // dx = dy = 0 exactly and adds fq * 0 = 0 (its mask is 0)
            keep = (own_lane && !self_in_stream) ? 0u : (all & ~p2p_mask[q]);
        }
        const unsigned ownm = __ballot_sync(full, own_lane);
        const int kown = (ownm && !self_in_stream) ? __ffs(ownm) - 1 : -1;
        // exclusive scan of the rows' kept counts; T = the stream's length
        const int c = __popc(keep);
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(full, incl, o);
            if (lane >= o) incl += t;
        }
        const int excl = incl - c, T = __shfl_sync(full, incl, 31);
        for (int k = 0; k < nq; k++) {
            const uint32_t mk = __shfl_sync(full, keep, k);
            const int ek = __shfl_sync(full, excl, k);
            if ((mk >> lane) & 1u) strm[w][ek + __popc(mk & lt)] = (uint16_t)((k << 5) | lane);
        }
        __syncwarp();
        const int32_t iA = t0 + tl, iB = t0 + tl + 16;
        const float4 mA = iA < t1 ? pos[iA] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 mB = iB < t1 ? pos[iB] : make_float4(0.f, 0.f, 0.f, 0.f);
        const uint64_t XA = pk2(mA.x, mA.x), YA = pk2(mA.y, mA.y), XB = pk2(mB.x, mB.x), YB = pk2(mB.y, mB.y);
        const uint64_t E2 = pk2(eps2, eps2);
        uint64_t AXA = 0, AYA = 0, AXB = 0, AYB = 0;
        float sxA = 0.f, syA = 0.f, sxB = 0.f, syB = 0.f;
        if (kown >= 0) {
            // the self row: gather, scalar, each half its own quads, the body itself excluded
            const int4 mo = meta[w][kown];
            const int j = mo.x + lane;
            const float4 v = j < mo.y ? pos[j] : far4;
            __syncwarp();
            sx[w][lane] = v.x;
            sy[w][lane] = v.y;
            sm[w][lane] = v.z;
            __syncwarp();
            const int ns = mo.y - mo.x;
            float xa, ya, xb, yb, d;
            upk2(XA, xa, d);
            upk2(YA, ya, d);
            upk2(XB, xb, d);
            upk2(YB, yb, d);
            for (int q = 0; q < 4; q++)
                for (int u = 0; u < 4; u++) {
                    const int kk = 8 * q + 4 * half + u;
                    if (kk >= ns) continue;
                    const float xj = sx[w][kk], yj = sy[w][kk], mj = sm[w][kk];
                    float dx = xj - xa, dy = yj - ya;
                    float ir = rsqrt_fast(fmaf(dx, dx, fmaf(dy, dy, eps2)));
                    float fk = mj * (ir * ir * ir);
                    fk = mo.x + kk == iA ? 0.f : fk;
                    sxA = fmaf(fk, dx, sxA);
                    syA = fmaf(fk, dy, syA);
                    dx = xj - xb;
                    dy = yj - yb;
                    ir = rsqrt_fast(fmaf(dx, dx, fmaf(dy, dy, eps2)));
                    fk = mj * (ir * ir * ir);
                    fk = mo.x + kk == iB ? 0.f : fk;
                    sxB = fmaf(fk, dx, sxB);
                    syB = fmaf(fk, dy, syB);
                }
        }
        // the stream, 32 sources at a time (this lane stages position ch * 32 + lane)
        auto fetch = [&](int p) -> float4 {
            if (p >= T) return far4;
            const int e = strm[w][p];
            const int4 mo = meta[w][e >> 5];
            float4 v = pos[mo.x + (e & 31)];
            v.x += __int_as_float(mo.z);
            v.y += __int_as_float(mo.w);
            return v;
        };
        const int nch = (T + 31) >> 5;
        float4 cur = nch > 0 ? fetch(lane) : far4;
        for (int ch = 0; ch < nch; ch++) {
            const float4 nxt = ch + 1 < nch ? fetch((ch + 1) * 32 + lane) : far4;
            __syncwarp();
            sx[w][lane] = cur.x;
            sy[w][lane] = cur.y;
            sm[w][lane] = cur.z;
            __syncwarp();
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int kk = 8 * q + 4 * half;
                float4 X = *reinterpret_cast<const float4 *>(&sx[w][kk]);
                float4 Y = *reinterpret_cast<const float4 *>(&sy[w][kk]);
                float4 Mq = *reinterpret_cast<const float4 *>(&sm[w][kk]);
                const uint64_t X0 = pk2(X.x, X.y), X1 = pk2(X.z, X.w), Y0 = pk2(Y.x, Y.y), Y1 = pk2(Y.z, Y.w);
                const uint64_t M0 = pk2(Mq.x, Mq.y), M1 = pk2(Mq.z, Mq.w);
                auto pair = [&](uint64_t XS, uint64_t YS, uint64_t MS, uint64_t XI, uint64_t YI, uint64_t &AX,
                                uint64_t &AY) {
                    uint64_t dx = sub2(XS, XI), dy = sub2(YS, YI);
                    uint64_t r = fma2(dx, dx, fma2(dy, dy, E2));
                    float ra, rb;
                    upk2(r, ra, rb);
                    uint64_t ir = pk2(rsqrt_fast(ra), rsqrt_fast(rb));
                    uint64_t fq = mul2(MS, mul2(mul2(ir, ir), ir));
                    AX = fma2(fq, dx, AX);
                    AY = fma2(fq, dy, AY);
                };
                pair(X0, Y0, M0, XA, YA, AXA, AYA);
                pair(X0, Y0, M0, XB, YB, AXB, AYB);
                pair(X1, Y1, M1, XA, YA, AXA, AYA);
                pair(X1, Y1, M1, XB, YB, AXB, AYB);
            }
            cur = nxt;
        }
        float a0, a1, b0, b1, c0, c1, e0, e1;
        upk2(AXA, a0, a1);
        upk2(AYA, b0, b1);
        upk2(AXB, c0, c1);
        upk2(AYB, e0, e1);
        float xA = (a0 + a1) + sxA, yA = (b0 + b1) + syA, xB = (c0 + c1) + sxB, yB = (e0 + e1) + syB;
        // the two halves hold the same targets over different sources: half 0 + half 1
        const float oxA = __shfl_xor_sync(full, xA, 16), oyA = __shfl_xor_sync(full, yA, 16);
        const float oxB = __shfl_xor_sync(full, xB, 16), oyB = __shfl_xor_sync(full, yB, 16);
        float2 res;
        if (half == 0) res = make_float2(xA + oxA, yA + oyA);  // target tl
        else res = make_float2(oxB + xB, oyB + yB);             // target tl + 16 (half 0's part first)
        part[it * 32 + lane] = res;
    }
}

// ---------------------------------------------------------------- M2P / P2L
// The leaf-level split of the ACCURATE near lists (theta_w > 0): a near leaf pair whose
// target bodies are all far from the source leaf takes the source's multipole at each
// target body (M2P, as extra work items of the target leaf, item_nq < 0); one whose
// source bodies are all far from the target leaf adds them to its local expansion (P2L,
// units of at most GX_P2L_UNIT source leaves).  Both use the unscaled Taylor
// coefficients a_k of 1/R, R^2 = dx^2 + dy^2 + eps^2, from the three-term recurrence of
// the fused M2L; a derivative of 1/R is k! a_k and the reference's G is its negative.

// a_k for |k| <= N at (dx, dy): a[gx_mi(k, l)]; NR = N or, above the unrolled orders, a
// run-time copy of it
template <int N, class T>
__device__ __forceinline__ void taylor_1r(T dx, T dy, T ir, T ir2, int NR, T *a) {
    a[0] = ir;
#pragma unroll
    for (int n = 1; n <= N; n++) {
        if (n > NR) break;
        const T in_ = tab_inv<T>(n) * ir2;
        const T c1 = -(T)(2 * n - 1) * in_, c2 = -(T)(n - 1) * in_;
        const T c1x = c1 * dx, c1y = c1 * dy;
#pragma unroll
        for (int k = 0; k <= n; k++) {
            const int l = n - k;
            T v;
            if (k >= 1 && l >= 1) v = c1x * a[gx_mi(k - 1, l)] + c1y * a[gx_mi(k, l - 1)];
            else if (k >= 1) v = c1x * a[gx_mi(k - 1, l)];
            else v = c1y * a[gx_mi(k, l - 1)];
            if (k >= 2) v += c2 * a[gx_mi(k - 2, l)];
            if (l >= 2) v += c2 * a[gx_mi(k, l - 2)];
            a[gx_mi(k, l)] = v;
        }
    }
}

// M2P of one source multipole M (about com_s, raw coefficients) at offset
// d = x - com_s:  a(x) = sum_S (-1)^|S| M[S] (S+e)! a_{S+e}(d), e = e_x, e_y.  FP32 at
// p >= 6 forms the coefficients at unit distance (the 1/R kernel is homogeneous of
// degree -1 in (d, eps)) and moves the powers of 1/R onto the moments, as the M2L does.
template <int P, class T>
__device__ __forceinline__ void m2p_eval(T dx, T dy, T eps2, const T *ms, T &fx, T &fy) {
    constexpr int N = P + 1;
    const int PP = gx_rt_order(P);
    const T ir = rsqrt_t<T>(dx * dx + dy * dy + eps2);
    T a[nc2(N)];
    T scale = T(1);
    T mw[nc2(P)];
    if constexpr (sizeof(T) == 4 && P >= 6) {
        T pw = T(1);
        for (int q = 0; q <= PP; q++) {
            for (int j = 0; j <= q; j++) mw[gx_mi(q - j, j)] = ms[gx_mi(q - j, j)] * pw;
            pw *= ir;
        }
        // at unit distance R' = 1: a'_0 = 1 and 1/R'^2 = 1 (eps enters through R only);
        // a_k(d) = a'_k(d / R) R^-(|k|+1)
        taylor_1r<N, T>(dx * ir, dy * ir, T(1), T(1), PP + 1, a);
        scale = ir * ir;
    } else {
#pragma unroll
        for (int k = 0; k < nc2(P); k++) mw[k] = ms[k];
        taylor_1r<N, T>(dx, dy, ir, ir * ir, PP + 1, a);
    }
    T sx = T(0), sy = T(0);
#pragma unroll
    for (int si = 0; si <= P; si++) {
        if (si > PP) break;
#pragma unroll
        for (int sj = 0; sj <= P - si; sj++) {
            if (si + sj > PP) break;
            const T mv = ((si + sj) & 1) ? -mw[gx_mi(si, sj)] : mw[gx_mi(si, sj)];
            sx += mv * (a[gx_mi(si + 1, sj)] * tab_ff<T>(si + 1, sj));
            sy += mv * (a[gx_mi(si, sj + 1)] * tab_ff<T>(si, sj + 1));
        }
    }
    fx += sx * scale;
    fy += sy * scale;
}

// M2P items: one warp per item with item_nq < 0 (grid-stride; P2P items are skipped),
// lane per target body (chunks of 32 above 32 bodies).  Per source leaf its lane forms
// the offset com_a - com_s in FP64 once (rounded to T), shared through shared memory;
// the source's moment row is a broadcast load.  Writes the item's partial slot like a
// P2P item, so the ordered sum of the leaf's items includes it.
template <int P, class T, class V>
__global__ void __launch_bounds__(128) k_m2p(int64_t n_list, const int32_t *__restrict__ list,
                                             const int32_t *__restrict__ item_leaf,
                                             const int64_t *__restrict__ item_qb, const int32_t *__restrict__ item_nq,
                                             const float4 *__restrict__ pos, const double *__restrict__ X,
                                             const double *__restrict__ Y, const double *__restrict__ comx,
                                             const double *__restrict__ comy, const int32_t *__restrict__ bs,
                                             const int32_t *__restrict__ be, const int32_t *__restrict__ src_idx,
                                             T eps2, const T *__restrict__ M, int tchunks, V *__restrict__ part) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    __shared__ T shx[4][32], shy[4][32];
    __shared__ int32_t shs[4][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t li = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; li < n_list; li += nwarps) {
        const int64_t it = list[li];
        const int nq0 = item_nq[it];
        if (nq0 >= 0) continue;
        const int nq = -nq0;
        const int32_t leaf = item_leaf[it];
        const double tcx = comx[leaf], tcy = comy[leaf];
        __syncwarp();  // the previous item's reads of the shared arrays are done
        if (lane < nq) {
            const int32_t sl = src_idx[item_qb[it] + lane];
            shs[w][lane] = sl;
            shx[w][lane] = (T)(tcx - comx[sl]);
            shy[w][lane] = (T)(tcy - comy[sl]);
        }
        __syncwarp();
        const int32_t t0 = bs[leaf], t1 = be[leaf];
        for (int tc = 0; tc < tchunks; tc++) {
            const int32_t i = t0 + tc * 32 + lane;
            T px = T(0), py = T(0);
            if (i < t1) {
                if constexpr (sizeof(T) == 4) {
                    const float4 v = pos[i];
                    px = v.x;
                    py = v.y;
                } else {
                    px = X[i] - tcx;
                    py = Y[i] - tcy;
                }
            }
            T fx = T(0), fy = T(0);
            if (t0 + tc * 32 < t1) {
                for (int k = 0; k < nq; k++) {
                    T ms[NC];
                    load_row<NC>(M + (int64_t)shs[w][k] * NS, ms);
                    m2p_eval<P, T>(px + shx[w][k], py + shy[w][k], eps2, ms, fx, fy);
                }
            }
            V r;
            r.x = fx;
            r.y = fy;
            part[(it * tchunks + tc) * 32 + lane] = r;
        }
    }
}

// Packed FP32 pairs (two bodies per lane) for the mixed-form M2P and P2L at p <= 5.
struct f2v {
    uint64_t v;
};
__device__ __forceinline__ f2v f2splat(float c) { return {pk2(c, c)}; }
__device__ __forceinline__ f2v f2pair(float a, float b) { return {pk2(a, b)}; }
__device__ __forceinline__ f2v f2mul(f2v a, f2v b) { return {mul2(a.v, b.v)}; }
__device__ __forceinline__ f2v f2add(f2v a, f2v b) { return {add2(a.v, b.v)}; }
__device__ __forceinline__ f2v f2sub(f2v a, f2v b) { return {sub2(a.v, b.v)}; }
__device__ __forceinline__ f2v f2fma(f2v a, f2v b, f2v c) { return {fma2(a.v, b.v, c.v)}; }

// taylor_1r on pairs: a_k for |k| <= N at two offsets at once
template <int N>
__device__ __forceinline__ void taylor_1r_x2(f2v dx, f2v dy, f2v ir, f2v ir2, f2v *a) {
    a[0] = ir;
#pragma unroll
    for (int n = 1; n <= N; n++) {
        const f2v in_ = f2mul(f2splat((float)(1.0 / n)), ir2);
        const f2v c1 = f2mul(f2splat(-(float)(2 * n - 1)), in_);
        const f2v c2 = f2mul(f2splat(-(float)(n - 1)), in_);
        const f2v c1x = f2mul(c1, dx), c1y = f2mul(c1, dy);
#pragma unroll
        for (int k = 0; k <= n; k++) {
            const int l = n - k;
            f2v v;
            if (k >= 1 && l >= 1) v = f2fma(c1x, a[gx_mi(k - 1, l)], f2mul(c1y, a[gx_mi(k, l - 1)]));
            else if (k >= 1) v = f2mul(c1x, a[gx_mi(k - 1, l)]);
            else v = f2mul(c1y, a[gx_mi(k, l - 1)]);
            if (k >= 2) v = f2fma(c2, a[gx_mi(k - 2, l)], v);
            if (l >= 2) v = f2fma(c2, a[gx_mi(k, l - 2)], v);
            a[gx_mi(k, l)] = v;
        }
    }
}

__device__ __forceinline__ f2v rsqrt_x2(f2v r2) {
    float a, b;
    upk2(r2.v, a, b);
    return f2pair(rsqrt_fast(a), rsqrt_fast(b));
}

// M2P items, mixed form, leaves of at most 32 bodies, p <= 5: lane tl of each half-warp
// holds target bodies tl and tl + 16 as a pair, half h takes the item's sources
// h, h + 2, ...; per source its lane stores the moments signed and scaled by (S+e)!
// (both components duplicated, ready as pair operands) and the COM offset in shared
// memory.  The halves' sums are added in a fixed order (half 0's first), as in the
// two-target P2P rows.
template <int P>
__global__ void __launch_bounds__(128, 8) k_m2p_x2(int64_t n_list, const int32_t *__restrict__ list,
                                                const int32_t *__restrict__ item_leaf,
                                                const int64_t *__restrict__ item_qb,
                                                const int32_t *__restrict__ item_nq, const float4 *__restrict__ pos,
                                                const double *__restrict__ comx, const double *__restrict__ comy,
                                                const int32_t *__restrict__ bs, const int32_t *__restrict__ be,
                                                const int32_t *__restrict__ src_idx, float eps2,
                                                const float *__restrict__ M, float2 *__restrict__ part) {
    static_assert(P <= 5, "shared-memory moment rows are sized for p <= 5");
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<float>(NC);
    __shared__ __align__(16) float4 smm[4][32][NC];  // (mx, mx, my, my) per moment
    __shared__ __align__(8) float2 shf[4][32];        // com_a - com_s
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int half = lane >> 4, tl = lane & 15;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const f2v E2 = f2splat(eps2);
    for (int64_t li = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; li < n_list; li += nwarps) {
        const int64_t it = list[li];
        const int nq0 = item_nq[it];
        if (nq0 >= 0) continue;
        const int nq = -nq0;
        const int32_t leaf = item_leaf[it];
        __syncwarp();  // the previous item's reads of the shared arrays are done
        if (lane < nq) {
            const int32_t sl = src_idx[item_qb[it] + lane];
            shf[w][lane] = make_float2((float)(comx[leaf] - comx[sl]), (float)(comy[leaf] - comy[sl]));
            float ms[NC];
            load_row<NC>(M + (int64_t)sl * NS, ms);
#pragma unroll
            for (int si = 0; si <= P; si++)
#pragma unroll
                for (int sj = 0; sj <= P - si; sj++) {
                    const float mv = ((si + sj) & 1) ? -ms[gx_mi(si, sj)] : ms[gx_mi(si, sj)];
                    const float mx = mv * tab_ff<float>(si + 1, sj), my = mv * tab_ff<float>(si, sj + 1);
                    smm[w][lane][gx_mi(si, sj)] = make_float4(mx, mx, my, my);
                }
        }
        __syncwarp();
        const int32_t t0 = bs[leaf], t1 = be[leaf];
        const int32_t iA = t0 + tl, iB = t0 + tl + 16;
        const float4 pA = iA < t1 ? pos[iA] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 pB = iB < t1 ? pos[iB] : make_float4(0.f, 0.f, 0.f, 0.f);
        const f2v X = f2pair(pA.x, pB.x), Y = f2pair(pA.y, pB.y);
        f2v FX = f2splat(0.f), FY = f2splat(0.f);
        for (int k = half; k < nq; k += 2) {
            const float2 o = shf[w][k];
            const f2v dx = f2add(X, f2splat(o.x)), dy = f2add(Y, f2splat(o.y));
            const f2v r2 = f2fma(dx, dx, f2fma(dy, dy, E2));
            const f2v ir = rsqrt_x2(r2);
            f2v a[nc2(P + 1)];
            taylor_1r_x2<P + 1>(dx, dy, ir, f2mul(ir, ir), a);
#pragma unroll
            for (int si = 0; si <= P; si++)
#pragma unroll
                for (int sj = 0; sj <= P - si; sj++) {
                    const float4 m4 = smm[w][k][gx_mi(si, sj)];
                    FX = f2fma(f2pair(m4.x, m4.y), a[gx_mi(si + 1, sj)], FX);
                    FY = f2fma(f2pair(m4.z, m4.w), a[gx_mi(si, sj + 1)], FY);
                }
        }
        float xA, xB, yA, yB;
        upk2(FX.v, xA, xB);
        upk2(FY.v, yA, yB);
        const float oxA = __shfl_xor_sync(0xffffffffu, xA, 16), oyA = __shfl_xor_sync(0xffffffffu, yA, 16);
        const float oxB = __shfl_xor_sync(0xffffffffu, xB, 16), oyB = __shfl_xor_sync(0xffffffffu, yB, 16);
        float2 res;
        if (half == 0) res = make_float2(xA + oxA, yA + oyA);  // body tl
        else res = make_float2(oxB + xB, oyB + yB);             // body tl + 16 (half 0's part first)
        part[it * 32 + lane] = res;
    }
}

// cp.async of 16 bytes global -> shared through L1 (a P2L source leaf is read by the
// units of many nearby target leaves), zero-filled when ok is false (no bytes are read
// then; src must still be a valid address)
__device__ __forceinline__ void cp_async16_zfill(void *dst_smem, const void *src, bool ok) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(ok ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
constexpr int P2L_RING = 4;  // rounds of P2L source bodies in flight per warp (three ahead)

// P2L units, mixed form, p <= 5: lane tl of each half-warp takes source bodies tl and
// tl + 16 of a source leaf as a pair, half h the unit's sources h, h + 2, ...; the
// coefficient sums stay pairs until the end (pair halves, then the warp, in a fixed
// order).  Leaves above 32 bodies go through their further bodies 32 at a time.
template <int P>
__global__ void __launch_bounds__(128, 6) k_p2l_x2(int64_t n_units, const int32_t *__restrict__ uleaf,
                                                const int64_t *__restrict__ ustart, const int32_t *__restrict__ ulen,
                                                const int64_t *__restrict__ leaf_u, const int64_t *__restrict__ body_u,
                                                const int32_t *__restrict__ src_idx, const float4 *__restrict__ pos,
                                                const double *__restrict__ comx, const double *__restrict__ comy,
                                                const int32_t *__restrict__ bs, const int32_t *__restrict__ be,
                                                float eps2, float *__restrict__ Lf, float *__restrict__ ppart) {
    static_assert(P <= 5, "paired accumulators are sized for p <= 5");
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<float>(NC);
    __shared__ __align__(16) float4 p2l_ring[4][P2L_RING][64];  // per warp: P2L_RING rounds x 64 bodies
    const int lane = threadIdx.x & 31;
    const int half = lane >> 4, tl = lane & 15;
    const int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (u >= n_units) return;
    const int32_t a = uleaf[u];
    const int nq = ulen[u];
    if (nq < 0) return;  // a body-level unit (k_p2l_body_x2)
    int32_t sb = 0, se = 0;
    float shx = 0.f, shy = 0.f;
    if (lane < nq) {
        const int32_t sl = src_idx[ustart[u] + lane];
        sb = bs[sl];
        se = be[sl];
        shx = (float)(comx[a] - comx[sl]);
        shy = (float)(comy[a] - comy[sl]);
    }
    const f2v E2 = f2splat(eps2);
    f2v acc[NC];
#pragma unroll
    for (int k = 0; k < NC; k++) acc[k] = f2splat(0.f);
    const int rounds = (nq + 1) >> 1;  // both halves run the same number of rounds
    // round r: this half's source k = 2r + half (its first 32 bodies: lane tl loads bodies
    // tl and tl + 16).  They are copied global -> shared by cp.async P2L_RING - 1 rounds
    // ahead, each lane reading back only its own copies, so the loads in flight hold no
    // registers; leaves above 32 bodies load the rest in place.
    auto src = [&](int r, int32_t &j0, int32_t &j1, float &ox, float &oy) {
        const int k = 2 * r + half;
        const int kk = k < nq ? k : 0;
        j0 = __shfl_sync(0xffffffffu, sb, kk);
        const int32_t e1 = __shfl_sync(0xffffffffu, se, kk);
        j1 = k < nq ? e1 : j0;  // the half without a source this round runs no body
        ox = __shfl_sync(0xffffffffu, shx, kk);
        oy = __shfl_sync(0xffffffffu, shy, kk);
    };
    auto body_pair = [&](const float4 &pA, const float4 &pB, float ox, float oy) {
        // com_a - x_j = (com_a - com_s) - (x_j - com_s); an empty slot has m = 0 and
        // sits at com_s, at the leaf pair's nonzero distance
        const f2v dx = f2sub(f2splat(ox), f2pair(pA.x, pB.x)), dy = f2sub(f2splat(oy), f2pair(pA.y, pB.y));
        const f2v ir = rsqrt_x2(f2fma(dx, dx, f2fma(dy, dy, E2)));
        f2v c[NC];
        taylor_1r_x2<P>(dx, dy, ir, f2mul(ir, ir), c);
        const f2v mm = f2pair(pA.z, pB.z);
#pragma unroll
        for (int q = 0; q < NC; q++) acc[q] = f2fma(mm, c[q], acc[q]);
    };
    float4 *ring = &p2l_ring[threadIdx.x >> 5][0][0];
    auto issue = [&](int r) {
        if (r < rounds) {
            int32_t j0, j1;
            float ox, oy;
            src(r, j0, j1, ox, oy);
            const int32_t jA = j0 + tl, jB = j0 + tl + 16;
            float4 *dst = ring + (r % P2L_RING) * 64 + lane;  // body A at lane, B at 32 + lane
            cp_async16_zfill(dst, pos + (jA < j1 ? jA : 0), jA < j1);
            cp_async16_zfill(dst + 32, pos + (jB < j1 ? jB : 0), jB < j1);
        }
        cp_async_commit();  // an empty group past the last round keeps the count uniform
    };
#pragma unroll
    for (int r = 0; r < P2L_RING - 1; r++) issue(r);
    for (int r = 0; r < rounds; r++) {
        issue(r + P2L_RING - 1);
        cp_async_wait<P2L_RING - 1>();  // round r's copies have landed
        int32_t c0, c1;
        float cox, coy;
        src(r, c0, c1, cox, coy);
        const float4 *slot = ring + (r % P2L_RING) * 64 + lane;
        if (c0 < c1) body_pair(slot[0], slot[32], cox, coy);
        for (int32_t b0 = c0 + 32; b0 < c1; b0 += 32) {
            const int32_t jA = b0 + tl, jB = b0 + tl + 16;
            const float4 pA = jA < c1 ? pos[jA] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 pB = jB < c1 ? pos[jB] : make_float4(0.f, 0.f, 0.f, 0.f);
            body_pair(pA, pB, cox, coy);
        }
    }
    cp_async_wait<0>();
    const bool single = (leaf_u[a + 1] - leaf_u[a]) + (body_u ? body_u[a + 1] - body_u[a] : 0) == 1;
#pragma unroll
    for (int q = 0; q < NC; q++) {
        float lo, hi;
        upk2(acc[q].v, lo, hi);
        const float v = warp_sum_t<float>(lo + hi);
        if (lane == (q & 31)) {
            if (single) Lf[(int64_t)a * NS + q] -= v;
            else ppart[u * NS + q] = v;
        }
    }
}

// Body-level P2L units, mixed form, p <= 5: a unit is up to GX_BODY_UNIT consecutive
// P2P rows (a <- s) of one target leaf with the plan's masks.  Each lane takes rows lane,
// lane + 32, ...: it loads the row, and after a warp scan of the rows' mask counts writes
// its masked bodies to the unit's stream in shared memory (entry (row << 5) | body, row
// and body order).  The stream is taken two bodies per lane, 64 at a time (positions
// c + lane and c + 32 + lane), each with its row's com_a - com_s; a padding slot has zero
// mass at a unit offset.  Writes like k_p2l_x2 (the leaf's units are summed in unit
// order, or a leaf with one unit subtracts its sum from its local directly).
template <int P>
__global__ void __launch_bounds__(128, 6) k_p2l_body_x2(int64_t u_base, int64_t n_units,
                                                     const int32_t *__restrict__ uleaf,
                                                     const int64_t *__restrict__ ustart,
                                                     const int32_t *__restrict__ ulen,
                                                     const int64_t *__restrict__ leaf_u,
                                                     const int64_t *__restrict__ body_u,
                                                     const int32_t *__restrict__ src_idx,
                                                     const uint32_t *__restrict__ p2p_mask,
                                                     const float4 *__restrict__ pos, const double *__restrict__ comx,
                                                     const double *__restrict__ comy, const int32_t *__restrict__ bs,
                                                     float eps2, float *__restrict__ Lf, float *__restrict__ ppart) {
    static_assert(P <= 5, "paired accumulators are sized for p <= 5");
    static_assert(GX_BODY_UNIT % 32 == 0 && GX_BODY_UNIT * 32 <= 65536, "whole rows per lane, 16-bit entries");
    constexpr int RPL = GX_BODY_UNIT / 32;  // rows per lane
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<float>(NC);
    __shared__ __align__(16) float2 rsh[4][GX_BODY_UNIT];  // per row: com_a - com_s in FP32
    __shared__ int32_t rb0[4][GX_BODY_UNIT];               // per row: the source leaf's first body
    __shared__ uint16_t strm[4][GX_BODY_UNIT * 32];        // the unit's masked bodies: (row << 5) | body
    const unsigned full = 0xffffffffu;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t wu = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (wu >= n_units) return;
    const int64_t u = u_base + wu;  // the body-level units follow the leaf-level ones
    const int raw = ulen[u];
    if (raw >= 0) return;  // a leaf-level unit (k_p2l_x2)
    const int nq = -raw;
    const int32_t a = uleaf[u];
    const double acx = comx[a], acy = comy[a];
    uint32_t take[RPL];
#pragma unroll
    for (int h = 0; h < RPL; h++) {
        take[h] = 0u;
        const int r = 32 * h + lane;
        if (r < nq) {
            const int64_t q = ustart[u] + r;
            const int32_t sl = src_idx[q];
            take[h] = p2p_mask[q];  // 0 for the self row
            rb0[w][r] = bs[sl];
            rsh[w][r] = make_float2((float)(acx - comx[sl]), (float)(acy - comy[sl]));
        }
    }
    // exclusive scan of the rows' counts (rows lane, then rows 32 + lane, ...)
    int base = 0, T = 0;
    int excl[RPL];
#pragma unroll
    for (int h = 0; h < RPL; h++) {
        const int c = __popc(take[h]);
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(full, incl, o);
            if (lane >= o) incl += t;
        }
        excl[h] = base + incl - c;
        base += __shfl_sync(full, incl, 31);
    }
    T = base;
#pragma unroll
    for (int h = 0; h < RPL; h++) {
        uint32_t m = take[h];
        int pp = excl[h];
        const int r = 32 * h + lane;
        while (m) {
            const int j = __ffs(m) - 1;
            m &= m - 1u;
            strm[w][pp++] = (uint16_t)((r << 5) | j);
        }
    }
    __syncwarp();
    const f2v E2 = f2splat(eps2);
    f2v acc[NC];
#pragma unroll
    for (int k = 0; k < NC; k++) acc[k] = f2splat(0.f);
    auto get = [&](int p, float4 &v, float2 &o) {
        if (p < T) {
            const int e = strm[w][p];
            v = pos[rb0[w][e >> 5] + (e & 31)];
            o = rsh[w][e >> 5];
        } else {
            v = make_float4(0.f, 0.f, 0.f, 0.f);
            o = make_float2(1.f, 1.f);
        }
    };
    float4 cA = make_float4(0.f, 0.f, 0.f, 0.f), cB = cA;
    float2 oA = make_float2(1.f, 1.f), oB = oA;
    if (T > 0) {
        get(lane, cA, oA);
        get(32 + lane, cB, oB);
    }
    for (int c0 = 0; c0 < T; c0 += 64) {
        float4 nA = make_float4(0.f, 0.f, 0.f, 0.f), nB = nA;
        float2 pA = make_float2(1.f, 1.f), pB = pA;
        if (c0 + 64 < T) {
            get(c0 + 64 + lane, nA, pA);
            get(c0 + 96 + lane, nB, pB);
        }
        // com_a - x_j = (com_a - com_s) - (x_j - com_s)
        const f2v dx = f2sub(f2pair(oA.x, oB.x), f2pair(cA.x, cB.x));
        const f2v dy = f2sub(f2pair(oA.y, oB.y), f2pair(cA.y, cB.y));
        const f2v ir = rsqrt_x2(f2fma(dx, dx, f2fma(dy, dy, E2)));
        f2v cf[NC];
        taylor_1r_x2<P>(dx, dy, ir, f2mul(ir, ir), cf);
        const f2v mm = f2pair(cA.z, cB.z);
#pragma unroll
        for (int q = 0; q < NC; q++) acc[q] = f2fma(mm, cf[q], acc[q]);
        cA = nA;
        cB = nB;
        oA = pA;
        oB = pB;
    }
    const bool single = (leaf_u[a + 1] - leaf_u[a]) + (body_u ? body_u[a + 1] - body_u[a] : 0) == 1;
#pragma unroll
    for (int q = 0; q < NC; q++) {
        float lo, hi;
        upk2(acc[q].v, lo, hi);
        const float v = warp_sum_t<float>(lo + hi);
        if (lane == (q & 31)) {
            if (single) Lf[(int64_t)a * NS + q] -= v;
            else ppart[u * NS + q] = v;
        }
    }
}

// P2L units: one warp per unit (a target leaf and at most GX_P2L_UNIT of its P2L source
// leaves), lane per source body.  L_a[T] += m_j G^(T)(com_a - x_j) / T! = -m_j a_T(com_a - x_j),
// summed per lane in body order, then over the warp; a leaf with one unit subtracts the
// sum from its local directly, otherwise the unit writes a partial and k_p2l_combine
// adds the partials in unit order.  Runs after L2L (the leaf locals exist) and before L2P.
// Lane q holds source q's body range and COM offset (one load round for the unit); the
// bodies of the next source are requested before the current ones are used.
template <int P, class T>
__device__ __forceinline__ void p2l_body(T dx, T dy, T mj, T eps2, T *acc) {
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    (void)NCr;
    const T ir = rsqrt_t<T>(dx * dx + dy * dy + eps2);
    T c[nc2(P)];
    if constexpr (sizeof(T) == 4 && P >= 6) {
        taylor_1r<P, T>(dx * ir, dy * ir, T(1), T(1), PP, c);
        T w = mj * ir;
        for (int q = 0; q <= PP; q++) {
            for (int i = 0; i <= q; i++) acc[gx_mi(q - i, i)] += w * c[gx_mi(q - i, i)];
            w *= ir;
        }
    } else {
        taylor_1r<P, T>(dx, dy, ir, ir * ir, PP, c);
#pragma unroll
        for (int k = 0; k < NCr; k++) acc[k] += mj * c[k];
    }
}

template <int P, class T>
__global__ void __launch_bounds__(128) k_p2l(int64_t n_units, const int32_t *__restrict__ uleaf,
                                             const int64_t *__restrict__ ustart, const int32_t *__restrict__ ulen,
                                             const int64_t *__restrict__ leaf_u, const int64_t *__restrict__ body_u,
                                             const int32_t *__restrict__ src_idx,
                                             const float4 *__restrict__ pos, const double *__restrict__ X,
                                             const double *__restrict__ Y, const double *__restrict__ Mb,
                                             const double *__restrict__ comx, const double *__restrict__ comy,
                                             const int32_t *__restrict__ bs, const int32_t *__restrict__ be, T eps2,
                                             const uint32_t *__restrict__ p2p_mask, int body_units,
                                             T *__restrict__ Lf, T *__restrict__ ppart) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    (void)NCr;
    const int lane = threadIdx.x & 31;
    const int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (u >= n_units) return;
    const int32_t a = uleaf[u];
    // a body-level unit (length stored negated): up to GX_BODY_UNIT P2P rows of the leaf,
    // their masked bodies only (source leaves of at most 32 bodies); body_units = 0 leaves
    // them to k_p2l_body_x2
    const int raw = ulen[u];
    if (raw < 0 && !body_units) return;
    const bool body = raw < 0;
    const int nq = body ? -raw : raw;
    const double tcx = comx[a], tcy = comy[a];
    T acc[NC];
#pragma unroll
    for (int k = 0; k < NCr; k++) acc[k] = T(0);
    // the unit's rows 32 at a time (a body-level unit has up to GX_BODY_UNIT)
    for (int g0 = 0; g0 < nq; g0 += 32) {
        const int ng = min(32, nq - g0);
        int32_t sb = 0, se = 0;
        uint32_t take = 0xffffffffu;
        T shx = T(0), shy = T(0);
        double scx = 0.0, scy = 0.0;
        if (lane < ng) {
            const int64_t q = ustart[u] + g0 + lane;
            if (body) take = p2p_mask[q];
            const int32_t sl = src_idx[q];
            sb = bs[sl];
            se = be[sl];
            scx = comx[sl];
            scy = comy[sl];
            shx = (T)(tcx - scx);
            shy = (T)(tcy - scy);
        }
        // one body of source k per lane (the first 32 of the leaf): relative position, mass
        auto fetch = [&](int k, T &px, T &py, T &pm) {
            const int32_t j = __shfl_sync(0xffffffffu, sb, k) + lane, j1 = __shfl_sync(0xffffffffu, se, k);
            if constexpr (sizeof(T) == 4) {
                const float4 v = j < j1 ? pos[j] : make_float4(0.f, 0.f, 0.f, 0.f);
                px = v.x;
                py = v.y;
                pm = v.z;
            } else {
                const double cx = __shfl_sync(0xffffffffu, scx, k), cy = __shfl_sync(0xffffffffu, scy, k);
                px = j < j1 ? X[j] - cx : 0.0;
                py = j < j1 ? Y[j] - cy : 0.0;
                pm = j < j1 ? Mb[j] : 0.0;
            }
        };
        T cx_ = T(0), cy_ = T(0), cm = T(0);
        fetch(0, cx_, cy_, cm);
        for (int k = 0; k < ng; k++) {
            T nx = T(0), ny = T(0), nm = T(0);
            if (k + 1 < ng) fetch(k + 1, nx, ny, nm);
            const T ox = __shfl_sync(0xffffffffu, shx, k), oy = __shfl_sync(0xffffffffu, shy, k);
            const int32_t j0 = __shfl_sync(0xffffffffu, sb, k), j1 = __shfl_sync(0xffffffffu, se, k);
            const double ckx = __shfl_sync(0xffffffffu, scx, k), cky = __shfl_sync(0xffffffffu, scy, k);
            (void)ckx;
            (void)cky;
            const uint32_t tk = __shfl_sync(0xffffffffu, take, k);
            // com_a - x_j = (com_a - com_s) - (x_j - com_s)
            if (j0 + lane < j1 && ((tk >> lane) & 1u)) p2l_body<P, T>(ox - cx_, oy - cy_, cm, eps2, acc);
            // leaves above 32 bodies (n_max > 32, never a body-level unit): the rest of the source's bodies
            for (int32_t j = j0 + 32 + lane; j < j1; j += 32) {
                T px, py, pm;
                if constexpr (sizeof(T) == 4) {
                    const float4 v = pos[j];
                    px = v.x;
                    py = v.y;
                    pm = v.z;
                } else {
                    px = X[j] - ckx;
                    py = Y[j] - cky;
                    pm = Mb[j];
                }
                p2l_body<P, T>(ox - px, oy - py, pm, eps2, acc);
            }
            cx_ = nx;
            cy_ = ny;
            cm = nm;
        }
    }
    const bool single = (leaf_u[a + 1] - leaf_u[a]) + (body_u ? body_u[a + 1] - body_u[a] : 0) == 1;
#pragma unroll
    for (int k = 0; k < NCr; k++) {
        const T v = warp_sum_t<T>(acc[k]);
        if (lane == (k & 31)) {
            if (single) Lf[(int64_t)a * NS + k] -= v;
            else ppart[u * NS + k] = v;
        }
    }
}

// Leaves with several P2L units: the partials in unit order, subtracted from the local.
template <int P, class T>
__global__ void k_p2l_combine(int64_t nl, const int64_t *__restrict__ leaf_u, const int64_t *__restrict__ body_u,
                              int64_t n_leafu, const T *__restrict__ ppart, T *__restrict__ Lf) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<T>(NC);
    const int PP = gx_rt_order(P);
    const int NCr = (PP + 1) * (PP + 2) / 2;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t a = t / NC;
    const int k = (int)(t - a * NC);
    if (a >= nl || k >= NCr) return;
    const int64_t u0 = leaf_u[a], u1 = leaf_u[a + 1];
    const int64_t b0 = body_u ? n_leafu + body_u[a] : 0, b1 = body_u ? n_leafu + body_u[a + 1] : 0;
    if ((u1 - u0) + (b1 - b0) < 2) return;
    T s = T(0);
    for (int64_t q = u0; q < u1; q++) s += ppart[q * NS + k];  // leaf-level units, then body-level ones
    for (int64_t q = b0; q < b1; q++) s += ppart[q * NS + k];
    Lf[a * NS + k] -= s;
}

// Folding of long item ranges.  A wide halo leaf can have ~1000 P2P items (977 at 1M
// Plummer, p = 4, n_max = 32, against a median of 5), and one warp summing them in
// order was the whole length of the reduce (its loads are dependent rounds of a few
// hundred cycles each).  So before the reduce, k_fold_items sums, in place, every full
// group of GX_FOLD items that starts at a multiple of GX_FOLD inside a leaf with more
// than GX_FOLD_MIN items; the reduce of such a leaf then reads its head items, the group
// sums and its tail items, in item order.  The groups depend only on the plan, so the
// sums are deterministic.
constexpr int GX_FOLD = 16, GX_FOLD_MIN = 32;

// The partial slots of a leaf's items [i0, i1): slot j < nh is item i0 + j, then ng group
// sums at h, h + GX_FOLD, ..., then the items [f, i1).  Unfolded leaves: nh = i1 - i0.
// Item indices fit in 31 bits (the partials of 2^31 items would take 512 GB).
struct ItemSlots {
    int i0, h, f, nh, ng, n;
    __device__ __forceinline__ ItemSlots(int64_t i0_, int64_t i1_) : i0((int)i0_) {
        const int i1 = (int)i1_;
        if (i1 - i0 > GX_FOLD_MIN) {
            h = (i0 + GX_FOLD - 1) / GX_FOLD * GX_FOLD;  // < i1: the leaf has more than 2 groups of items
            f = i1 / GX_FOLD * GX_FOLD;                  // >= h for the same reason
        } else {
            h = f = i1;
        }
        nh = h - i0;
        ng = (f - h) / GX_FOLD;
        n = nh + ng + (i1 - f);
    }
    __device__ __forceinline__ int operator[](int j) const {
        return j < nh ? i0 + j : (j < nh + ng ? h + (j - nh) * GX_FOLD : f + (j - nh - ng));
    }
};

__device__ __forceinline__ void vadd(float2 &a, const float2 &b) { a.x += b.x; a.y += b.y; }
__device__ __forceinline__ void vadd(double2 &a, const double2 &b) { a.x += b.x; a.y += b.y; }
__device__ __forceinline__ void vadd(float4 &a, const float4 &b) { a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w; }
__device__ __forceinline__ void vadd(double4 &a, const double4 &b) { a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w; }

// One warp per group of GX_FOLD items starting at a multiple of GX_FOLD; only groups
// wholly inside a leaf with more than GX_FOLD_MIN items are summed (into the group's
// first slot, for every target chunk): u and u + 8 pairwise, then a fixed tree.
template <class V>
__global__ void __launch_bounds__(128) k_fold_items(int64_t n_items, const int32_t *__restrict__ item_leaf,
                                                    const int64_t *__restrict__ item_off, int tchunks,
                                                    V *__restrict__ part) {
    static_assert(GX_FOLD == 16, "the sum below is written for groups of 16");
    const int lane = threadIdx.x & 31;
    const int64_t g0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * GX_FOLD;
    if (g0 >= n_items) return;
    const int32_t leaf = item_leaf[g0];
    const int64_t i0 = item_off[leaf], i1 = item_off[leaf + 1];
    if (i1 - i0 <= GX_FOLD_MIN || g0 + GX_FOLD > i1) return;
    for (int tc = 0; tc < tchunks; tc++) {
        V a[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            a[u] = part[((g0 + u) * tchunks + tc) * 32 + lane];
            vadd(a[u], part[((g0 + 8 + u) * tchunks + tc) * 32 + lane]);
        }
        vadd(a[0], a[1]);
        vadd(a[2], a[3]);
        vadd(a[4], a[5]);
        vadd(a[6], a[7]);
        vadd(a[0], a[2]);
        vadd(a[4], a[6]);
        vadd(a[0], a[4]);
        part[(g0 * tchunks + tc) * 32 + lane] = a[0];
    }
}

// Sum of a leaf's P2P partials over its item slots for one lane: eight independent
// accumulators (slot j into accumulator j mod 8), and the last (or only: the median
// leaf has 5 items) round of fewer than eight slots predicated rather than looped, so
// that the loads of a round are in flight together.
template <class V, class S>
__device__ __forceinline__ void sum_items(const V *__restrict__ part, int64_t i0, int64_t i1, int tchunks, int tc,
                                          int lane, S &sx, S &sy) {
    S ax[8] = {0, 0, 0, 0, 0, 0, 0, 0}, ay[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const ItemSlots sl(i0, i1);
    const V *base = part + tc * 32 + lane;
    const int64_t row = (int64_t)tchunks * 32;
    int j = 0;
    for (; j + 8 <= sl.n; j += 8) {
#pragma unroll
        for (int u = 0; u < 8; u++) {
            V v = base[sl[j + u] * row];
            ax[u] += v.x;
            ay[u] += v.y;
        }
    }
    if (j < sl.n) {
        const int r = sl.n - j;
        V v[8];
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (u < r) v[u] = base[sl[j + u] * row];
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (u < r) {
                ax[u] += v[u].x;
                ay[u] += v[u].y;
            }
    }
    sx = ((ax[0] + ax[1]) + (ax[2] + ax[3])) + ((ax[4] + ax[5]) + (ax[6] + ax[7]));
    sy = ((ay[0] + ay[1]) + (ay[2] + ay[3])) + ((ay[4] + ay[5]) + (ay[6] + ay[7]));
}

template <int P>
__global__ void __launch_bounds__(128) k_l2p_reduce64(int64_t nl, const double *__restrict__ x, const double *__restrict__ y,
                                                      const double *__restrict__ comx, const double *__restrict__ comy,
                                                      const int32_t *__restrict__ bs, const int32_t *__restrict__ be,
                                                      const double *__restrict__ Lf, const int64_t *__restrict__ item_off,
                                                      int tchunks, const double2 *__restrict__ part,
                                                      double *__restrict__ ax, double *__restrict__ ay,
                                                      double *__restrict__ hax, double *__restrict__ hay) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<double>(NC);
    int lane = threadIdx.x & 31;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (leaf >= nl) return;
    int32_t t0 = bs[leaf], t1 = be[leaf];
    int64_t i0 = item_off[leaf], i1 = item_off[leaf + 1];
    for (int tc = 0; tc < tchunks && t0 + tc * 32 < t1; tc++) {
        int32_t i = t0 + tc * 32 + lane;
        if (i >= t1) continue;
        double fx, fy;
        l2p_eval<P, double>(Lf + leaf * NS, x[i] - comx[leaf], y[i] - comy[leaf], fx, fy);
        double sx, sy;
        sum_items<double2, double>(part, i0, i1, tchunks, tc, lane, sx, sy);
        ax[i] = sx - fx;
        ay[i] = sy - fy;
        if (hax) {
            hax[i] = sx - fx;
            hay[i] = sy - fy;
        }
    }
}

// Mixed form, in two kernels: the L2P of every body on the main stream while the near
// field still runs (fl = the local expansion's (fx, fy) in FP32), and after the join the
// ordered sum of the P2P partials, a = sum - f in FP64.  The sum kernel has nothing but
// its loads to wait for, so more of its warps are resident and its loads (the leaf's
// item range, then the partials and fl together) are two dependent rounds.
template <int P>
__global__ void __launch_bounds__(128) k_l2p32(int64_t nl, const float4 *__restrict__ pos,
                                               const int32_t *__restrict__ bs, const int32_t *__restrict__ be,
                                               const float *__restrict__ Lf, float2 *__restrict__ fl) {
    constexpr int NC = nc2(P);
    constexpr int NS = row_stride<float>(NC);
    int lane = threadIdx.x & 31;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (leaf >= nl) return;
    int32_t t0 = bs[leaf], t1 = be[leaf];
    for (int32_t i = t0 + lane; i < t1; i += 32) {
        float4 me = pos[i];
        float fx, fy;
        l2p_eval<P, float>(Lf + leaf * NS, me.x, me.y, fx, fy);
        fl[i] = make_float2(fx, fy);
    }
}

__global__ void __launch_bounds__(128) k_reduce32(int64_t nl, const int32_t *__restrict__ bs,
                                                  const int32_t *__restrict__ be, const int64_t *__restrict__ item_off,
                                                  int tchunks, const float2 *__restrict__ part,
                                                  const float2 *__restrict__ fl, double *__restrict__ ax,
                                                  double *__restrict__ ay, double *__restrict__ hax,
                                                  double *__restrict__ hay) {
    int lane = threadIdx.x & 31;
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (leaf >= nl) return;
    int32_t t0 = bs[leaf], t1 = be[leaf];
    int64_t i0 = item_off[leaf], i1 = item_off[leaf + 1];
    for (int tc = 0; tc < tchunks && t0 + tc * 32 < t1; tc++) {
        int32_t i = t0 + tc * 32 + lane;
        if (i >= t1) continue;
        const float2 f = fl[i];
        float sx, sy;
        sum_items<float2, float>(part, i0, i1, tchunks, tc, lane, sx, sy);
        const double rx = (double)sx - (double)f.x, ry = (double)sy - (double)f.y;
        ax[i] = rx;
        ay[i] = ry;
        if (hax) {  // the caller's page-locked arrays, written over the host link as the sums finish
            hax[i] = rx;
            hay[i] = ry;
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
    if (ctx->in_x)
        k_prepare_from<<<gx_blocks(n, 256), 256, 0, st>>>(n, ctx->in_x, ctx->in_y, ctx->in_m, dptr<double>(ctx->x),
                                                          dptr<double>(ctx->y), dptr<double>(ctx->m), dptr<double>(ctx->ax),
                                                          dptr<double>(ctx->ay), dptr<unsigned>(ctx->status));
    else
        k_prepare<<<gx_blocks(n, 256), 256, 0, st>>>(n, dptr<double>(ctx->x), dptr<double>(ctx->y), dptr<double>(ctx->m),
                                                     dptr<double>(ctx->ax), dptr<double>(ctx->ay), dptr<unsigned>(ctx->status));
    ctx->launches++;
    tm.mark();  // 1
    if (nn == 0) {
        GX_CUDA(ctx, cudaGetLastError());
        ctx->last_launches = ctx->launches - launches0;
        return GX_OK;
    }
    const double *X = dptr<double>(ctx->x), *Y = dptr<double>(ctx->y), *Mb = dptr<double>(ctx->m);
    const double *comx = dptr<double>(ctx->comx), *comy = dptr<double>(ctx->comy);
    const int32_t *bs = dptr<int32_t>(ctx->bs), *be = dptr<int32_t>(ctx->be), *parent = dptr<int32_t>(ctx->parent);
    const int4 *child = dptr<int4>(ctx->child);
    const unsigned gw = (unsigned)((nl * 32 + 127) / 128);  // warp per leaf
    const double eps2 = ctx->eps * ctx->eps;
    const gx_ctx::Items &I = mode == GX_MODE_ACCURATE ? ctx->items_acc : ctx->items_ref;
    const int tchunks = (int)std::max<int64_t>(1, (ctx->max_leaf + 31) / 32);
    const int32_t *src_idx = mode == GX_MODE_ACCURATE ? dptr<int32_t>(ctx->near_idx) : dptr<int32_t>(ctx->p2p_idx);
    const unsigned gi = (unsigned)((I.n * 32 + 127) / 128);  // warp per item
    const bool split = mode == GX_MODE_ACCURATE && ctx->theta_w > 0.0;  // near-list split: M2P items, P2L units
    // body-level P2L of the P2P rows: masks in the plan, body-level P2L units
    const bool body = split && ctx->plan_body_split && gx_body_split_on(ctx);
    const uint32_t *p2p_mask = body ? dptr<uint32_t>(ctx->p2p_mask) : nullptr;

    auto passes = [&](auto tag) -> int {
        using T = decltype(tag);
        DevBuf &Mb_ = mixed ? ctx->Mf32 : ctx->M;
        DevBuf &Lb_ = mixed ? ctx->Lf32 : ctx->L;
        DevBuf &Lfb_ = mixed ? ctx->Lff32 : ctx->Lf;
        constexpr int NS = row_stride<T>(NC);
        GX_TRY(gx_ensure(ctx, Mb_, sizeof(T) * NS * (size_t)nn));
        GX_TRY(gx_ensure(ctx, Lb_, sizeof(T) * NS * (size_t)nn));
        GX_TRY(gx_ensure(ctx, Lfb_, sizeof(T) * NS * (size_t)nl));
        T *M = dptr<T>(Mb_), *L = dptr<T>(Lb_), *Lf = dptr<T>(Lfb_);
        float4 *pos = nullptr;
        if (mixed) {
            GX_TRY(gx_ensure(ctx, ctx->pos32, sizeof(float4) * (size_t)n));
            pos = dptr<float4>(ctx->pos32);
        }
        // P2M (+ FP32 body packing in the mixed form)
        k_p2m<P, T><<<gw, 128, 0, st>>>(nl, X, Y, Mb, comx, comy, bs, be, M, pos);
        ctx->launches++;
        tm.mark();  // 2
        // near field on the second stream, beside M2M -> M2L -> L2L on this one: both
        // are FP32-pipe bound but neither fills it alone (latency, occupancy), and
        // their blocks share the SMs.  Deterministic: P2P writes per-item partials
        // that L2P sums in order after the join.
        const size_t pbytes = (mixed ? sizeof(float2) : sizeof(double2)) * 32 * (size_t)tchunks * (size_t)(I.n + 1);
        GX_TRY(gx_ensure(ctx, ctx->part, pbytes));
        auto near_field = [&]() -> int {
        GX_CUDA(ctx, cudaEventRecord(ctx->ev_fork, st));
        GX_CUDA(ctx, cudaStreamWaitEvent(ctx->stream2, ctx->ev_fork, 0));
        if (timed) GX_CUDA(ctx, cudaEventRecord(ctx->ev[14], ctx->stream2));
        if (I.n > 0) {
            // two targets per lane pays when leaves fill most of a row; with leaves of at
            // most 16 bodies (n_max <= 16) the second target would be empty
            if (mixed && body)
                k_p2p32_stream<<<gi, 128, 0, ctx->stream2>>>(I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb),
                                                             dptr<int32_t>(I.nq), pos, comx, comy, bs, be, src_idx,
                                                             p2p_mask, (float)eps2, dptr<float2>(ctx->part));
            else if (mixed && tchunks == 1 && ctx->max_leaf <= 16)
                k_p2p32_rows1<<<gi, 128, 0, ctx->stream2>>>(I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb),
                                                            dptr<int32_t>(I.nq), pos, comx, comy, bs, be, src_idx,
                                                            (float)eps2, dptr<float2>(ctx->part));
            else if (mixed && tchunks == 1)
                k_p2p32_rows<<<gi, 128, 0, ctx->stream2>>>(I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb),
                                                           dptr<int32_t>(I.nq), pos, comx, comy, bs, be, src_idx,
                                                           (float)eps2, dptr<float2>(ctx->part));
            else if (mixed)
                k_p2p32_items<<<gi, 128, 0, ctx->stream2>>>(I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb),
                                                            dptr<int32_t>(I.nq), pos, comx, comy, bs, be, src_idx,
                                                            (float)eps2, tchunks, dptr<float2>(ctx->part));
            else
                k_p2p64_items<<<gi, 128, 0, ctx->stream2>>>(I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb),
                                                            dptr<int32_t>(I.nq), X, Y, Mb, bs, be, src_idx, p2p_mask, eps2,
                                                            tchunks, dptr<double2>(ctx->part));
            ctx->launches++;
        }
        if (timed) GX_CUDA(ctx, cudaEventRecord(ctx->ev[15], ctx->stream2));  // the P2P kernel alone
        if (split && ctx->n_m2p_items > 0) {
            const unsigned gm = (unsigned)((ctx->n_m2p_items * 32 + 127) / 128);  // warp per M2P item
            // M2P items of the near-list split: their own slots of the same partial array
            if constexpr (P <= 5) {
                if (mixed && tchunks == 1) {
                    k_m2p_x2<P><<<gm, 128, 0, ctx->stream2>>>(ctx->n_m2p_items, dptr<int32_t>(ctx->m2p_list),
                                                              dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb),
                                                              dptr<int32_t>(I.nq), pos, comx, comy, bs, be, src_idx,
                                                              (float)eps2, reinterpret_cast<const float *>(M),
                                                              dptr<float2>(ctx->part));
                    goto m2p_done;
                }
            }
            if (mixed)
                k_m2p<P, float, float2><<<gm, 128, 0, ctx->stream2>>>(
                    ctx->n_m2p_items, dptr<int32_t>(ctx->m2p_list), dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb), dptr<int32_t>(I.nq), pos, nullptr, nullptr, comx,
                    comy, bs, be, src_idx, (float)eps2, reinterpret_cast<const float *>(M), tchunks,
                    dptr<float2>(ctx->part));
            else
                k_m2p<P, double, double2><<<gm, 128, 0, ctx->stream2>>>(
                    ctx->n_m2p_items, dptr<int32_t>(ctx->m2p_list), dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb), dptr<int32_t>(I.nq), nullptr, X, Y, comx, comy, bs,
                    be, src_idx, eps2, reinterpret_cast<const double *>(M), tchunks, dptr<double2>(ctx->part));
        m2p_done:
            ctx->launches++;
        }
        if (I.n > GX_FOLD_MIN) {
            const unsigned gf = (unsigned)(((I.n + GX_FOLD - 1) / GX_FOLD * 32 + 127) / 128);
            if (mixed)
                k_fold_items<float2><<<gf, 128, 0, ctx->stream2>>>(I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.off),
                                                                   tchunks, dptr<float2>(ctx->part));
            else
                k_fold_items<double2><<<gf, 128, 0, ctx->stream2>>>(I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.off),
                                                                    tchunks, dptr<double2>(ctx->part));
            ctx->launches++;
        }
        GX_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->stream2));
        return GX_OK;
        };
        // the near field starts beside the far-field chain; for a measurement of the
        // near field alone (gx_bench_forces) it starts after the chain
        if (!ctx->near_after_far) GX_TRY(near_field());
        // M2M, bottom-up by level; in ACCURATE mode the single-child chain levels over the
        // leaves are one direct shift (their nodes have no far lists)
        int lv_m2m = 1;
        if (mode == GX_MODE_ACCURATE && ctx->chain_levels >= 2) {
            const int64_t up = ctx->level_start[ctx->chain_levels];
            k_m2m_chain<P, T><<<gx_blocks(nl, 128), 128, 0, st>>>(nl, up, comx, comy, M);
            ctx->launches++;
            lv_m2m = ctx->chain_levels + 1;
        }
        for (int lv = lv_m2m; lv < ctx->n_levels; lv++) {
            int64_t s = ctx->level_start[lv], e = ctx->level_start[lv + 1];
            k_m2m<P, T><<<gx_blocks(e - s, 128), 128, 0, st>>>(s, e, child, comx, comy, M);
            ctx->launches++;
        }
        if (ctx->n_levels > 1) {
            k_scrub<T><<<gx_blocks(NS * nn, 256), 256, 0, st>>>(NS * nn, M);
            ctx->launches++;
        }
        tm.mark();  // 3
        // M2L
        const unsigned gn = (unsigned)((nn * 32 + 127) / 128);
        if (mode == GX_MODE_REF && !mixed) {
            k_m2l_ref<P><<<gn, 128, 0, st>>>(nn, dptr<uint32_t>(ctx->vdata), dptr<uint8_t>(ctx->vlen),
                                             dptr<int64_t>(ctx->ref_voff), dptr<int32_t>(ctx->ref_did),
                                             dptr<double>(ctx->ref_G), reinterpret_cast<const double *>(M),
                                             reinterpret_cast<double *>(L));
        } else if (mode == GX_MODE_ACCURATE) {
            // nodes without far sources keep whatever L holds: has_far = 0 keeps L2L from reading it
            const gx_ctx::M2LUnits &U = ctx->m2l_units;
            GX_TRY(gx_ensure(ctx, ctx->m2l_part, sizeof(T) * NS * (size_t)(U.n + 1)));
            if (U.n > 0) {
                const int64_t *node_u = dptr<int64_t>(U.node_u);
                k_m2l_units<P, T><<<(unsigned)((U.n * 32 + 127) / 128), 128, 0, st>>>(
                    U.n, dptr<int32_t>(U.node), dptr<int64_t>(U.start), dptr<int32_t>(U.len), node_u,
                    dptr<int32_t>(ctx->far_idx), comx, comy, mixed ? dptr<float4>(ctx->comhl) : nullptr, eps2, M, L,
                    dptr<T>(ctx->m2l_part));
                k_m2l_combine<P, T><<<gx_blocks(nn * NC, 256), 256, 0, st>>>(nn, node_u, dptr<T>(ctx->m2l_part), L);
                ctx->launches++;
            }
        } else {
            k_m2l_exact<P, T, uint32_t><<<gn, 128, 0, st>>>(nn, dptr<uint32_t>(ctx->vdata), nullptr, nullptr,
                                                            dptr<uint8_t>(ctx->vlen), GX_LIST_CAP, comx, comy,
                                                            mixed ? dptr<float4>(ctx->comhl) : nullptr, eps2, M, L);
        }
        ctx->launches++;
        tm.mark();  // 4
        // L2L
        const T *Lleaf = L;
        if (mode == GX_MODE_REF) {
            k_l2l_ref_leaves<P, T><<<gx_blocks(nl, 128), 128, 0, st>>>(nl, parent, comx, comy, L, Lf);
            ctx->launches++;
            Lleaf = Lf;
        } else {
            k_l2l_direct<P, T><<<gw, 128, 0, st>>>(nl, ctx->n_levels, dptr<int32_t>(ctx->anc),
                                                   dptr<uint8_t>(mode == GX_MODE_ACCURATE ? ctx->has_far_acc
                                                                                          : ctx->has_far_ref),
                                                   comx, comy, L, Lf);
            ctx->launches++;
            Lleaf = Lf;
        }
        if (split && ctx->p2l_units.n > 0) {
            // P2L of the near-list split into the leaf locals, before L2P reads them
            const gx_ctx::P2LUnits &PU = ctx->p2l_units;
            GX_TRY(gx_ensure(ctx, ctx->p2l_part, sizeof(T) * NS * (size_t)(PU.n + 1)));
            const int64_t *leaf_u = dptr<int64_t>(PU.leaf_u);
            const int64_t *body_u = body ? dptr<int64_t>(PU.body_u) : nullptr;
            const unsigned gu = (unsigned)((PU.n * 32 + 127) / 128);
            const unsigned gl = (unsigned)((PU.n_leafu * 32 + 127) / 128);
            const unsigned gb = (unsigned)((PU.n_body * 32 + 127) / 128);
            bool packed = false;
            if constexpr (P <= 5 && sizeof(T) == 4) {
                // leaf-level units, then (body-level P2L) the body-level ones
                if (PU.n_leafu > 0)
                    k_p2l_x2<P><<<gl, 128, 0, st>>>(PU.n_leafu, dptr<int32_t>(PU.leaf), dptr<int64_t>(PU.start),
                                                    dptr<int32_t>(PU.len), leaf_u, body_u, src_idx, pos, comx, comy,
                                                    bs, be, (float)eps2, Lf, dptr<float>(ctx->p2l_part));
                if (body && PU.n_body > 0) {
                    k_p2l_body_x2<P><<<gb, 128, 0, st>>>(PU.n_leafu, PU.n_body, dptr<int32_t>(PU.leaf),
                                                         dptr<int64_t>(PU.start), dptr<int32_t>(PU.len), leaf_u,
                                                         body_u, src_idx, p2p_mask, pos, comx, comy, bs, (float)eps2,
                                                         Lf, dptr<float>(ctx->p2l_part));
                    ctx->launches++;
                }
                packed = true;
            }
            if (!packed)
                k_p2l<P, T><<<gu, 128, 0, st>>>(PU.n, dptr<int32_t>(PU.leaf), dptr<int64_t>(PU.start),
                                                dptr<int32_t>(PU.len), leaf_u, body_u, src_idx, pos, X, Y, Mb, comx,
                                                comy, bs, be, (T)eps2, p2p_mask, body ? 1 : 0, Lf,
                                                dptr<T>(ctx->p2l_part));
            k_p2l_combine<P, T><<<gx_blocks(nl * NC, 256), 256, 0, st>>>(nl, leaf_u, body_u, PU.n_leafu,
                                                                         dptr<T>(ctx->p2l_part), Lf);
            ctx->launches += 2;
        }
        float2 *fl = nullptr;
        if (mixed) {  // L2P beside the near field
            GX_TRY(gx_ensure(ctx, ctx->fl32, sizeof(float2) * (size_t)n));
            fl = dptr<float2>(ctx->fl32);
            k_l2p32<P><<<gw, 128, 0, st>>>(nl, pos, bs, be, reinterpret_cast<const float *>(Lleaf), fl);
            ctx->launches++;
        }
        tm.mark();  // 5
        if (ctx->near_after_far) GX_TRY(near_field());
        // join the near field, then the ordered sum of the P2P partials (+ L2P in FP64)
        GX_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_join, 0));
        if (mixed) {
            k_reduce32<<<gw, 128, 0, st>>>(nl, bs, be, dptr<int64_t>(I.off), tchunks, dptr<float2>(ctx->part), fl,
                                           dptr<double>(ctx->ax), dptr<double>(ctx->ay), ctx->out_ax, ctx->out_ay);
        } else {
            k_l2p_reduce64<P><<<gw, 128, 0, st>>>(nl, X, Y, comx, comy, bs, be, reinterpret_cast<const double *>(Lleaf),
                                                  dptr<int64_t>(I.off), tchunks, dptr<double2>(ctx->part),
                                                  dptr<double>(ctx->ax), dptr<double>(ctx->ay), ctx->out_ax,
                                                  ctx->out_ay);
        }
        ctx->launches++;
        tm.mark();  // 6
        return GX_OK;
    };
    if (mixed) {
        GX_TRY(passes(float{}));
    } else {
        GX_TRY(passes(double{}));
    }
    GX_CUDA(ctx, cudaGetLastError());
    ctx->last_launches = ctx->launches - launches0;
    return GX_OK;
}

}  // namespace

#define GX_FMM_INSTANTIATE(PP) \
    int gx_run_forces_##PP(gx_ctx *ctx, bool timed) { return run_forces<PP>(ctx, timed); }
