// gx_scan.cu -- device-wide exclusive scan and a stable LSD radix sort.
//
// The radix sort replaces the stable `indices.sort_by_key(|&i| keys[i])` of
// Tree::build (galax-core/src/lib.rs:192).  It is a three-kernel
// reduce-then-scan design: no kernel waits on another CTA, so there is no
// inter-block spin anywhere.  Stability: within a tile each warp owns a
// contiguous run of 256 items and ranks them in index order with
// __match_any_sync; warps and tiles are ordered by the digit-major offset scan.
#include "gx_internal.cuh"

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // 1024

template <class T>
__device__ T block_exclusive_scan(T v, T *total) {
    __shared__ T warp_tot[SCAN_THREADS / 32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
        T s = (lane < SCAN_THREADS / 32) ? warp_tot[lane] : T(0);
        T si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T t = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= o) si += t;
        }
        if (lane < SCAN_THREADS / 32) warp_tot[lane] = si - s;
        if (lane == SCAN_THREADS / 32 - 1) *total = si;
    }
    __syncthreads();
    T r = warp_tot[w] + inc - v;
    __syncthreads();
    return r;
}

template <class T>
__global__ void k_scan_sums(const T *in, int64_t n, T *sums) {
    __shared__ T tot;
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    T s = 0;
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
        if (i < n) s += in[i];
    }
    block_exclusive_scan<T>(s, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// In-place exclusive scan of `sums` (nb entries) by one block; writes the grand total.
template <class T>
__device__ void scan_single_block(T *sums, int64_t nb, T *total) {
    __shared__ T tot;
    T carry = 0;
    for (int64_t base = 0; base < nb; base += SCAN_TILE) {
        T v[SCAN_ITEMS];
        T s = 0;
        for (int k = 0; k < SCAN_ITEMS; k++) {
            int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
            v[k] = (i < nb) ? sums[i] : T(0);
            s += v[k];
        }
        T ex = block_exclusive_scan<T>(s, &tot);
        T run = carry + ex;
        for (int k = 0; k < SCAN_ITEMS; k++) {
            int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
            if (i < nb) sums[i] = run;
            run += v[k];
        }
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

template <class T>
__global__ void k_scan_single(T *sums, int64_t nb, T *total) {
    scan_single_block<T>(sums, nb, total);
}

template <class T>
__global__ void k_scan_apply(const T *in, T *out, int64_t n, const T *sums) {
    __shared__ T tot;
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    T v[SCAN_ITEMS];
    T s = 0;
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
        v[k] = (i < n) ? in[i] : T(0);
        s += v[k];
    }
    T run = sums[blockIdx.x] + block_exclusive_scan<T>(s, &tot);
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
}

// Device-length forms: the length is *n_dev + n_add (at most n_cap), read on the
// device, so a scan over a count produced by an earlier kernel needs no host round
// trip.  Grids are sized for n_cap; blocks past the length do no work.
__device__ __forceinline__ int64_t dev_len(const int64_t *n_dev, int64_t n_add, int64_t n_cap) {
    int64_t n = *n_dev + n_add;
    return n < n_cap ? n : n_cap;
}

// blockIdx.y selects one of gridDim.y arrays: in + y * stride, out + y * stride, and
// the block sums of array y at sums + y * (gridDim.x + 1)
__global__ void k_scan_sums_dn(const int64_t *in, const int64_t *n_dev, int64_t n_add, int64_t n_cap, int64_t *sums,
                               int64_t stride) {
    __shared__ int64_t tot;
    const int64_t n = dev_len(n_dev, n_add, n_cap);
    in += blockIdx.y * stride;
    sums += blockIdx.y * (int64_t)(gridDim.x + 1);
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int64_t s = 0;
    if (base < n)
        for (int k = 0; k < SCAN_ITEMS; k++) {
            int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
            if (i < n) s += in[i];
        }
    block_exclusive_scan<int64_t>(s, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_single_dn(int64_t *sums, int64_t nb, int64_t *total) {
    const int64_t y = blockIdx.x;
    scan_single_block<int64_t>(sums + y * (nb + 1), nb, total ? total + y : sums + y * (nb + 1) + nb);
}

__global__ void k_scan_apply_dn(const int64_t *in, int64_t *out, const int64_t *n_dev, int64_t n_add, int64_t n_cap,
                                const int64_t *sums, int64_t stride) {
    __shared__ int64_t tot;
    const int64_t n = dev_len(n_dev, n_add, n_cap);
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    if (base >= n) return;  // uniform per block
    in += blockIdx.y * stride;
    out += blockIdx.y * stride;
    sums += blockIdx.y * (int64_t)(gridDim.x + 1);
    int64_t v[SCAN_ITEMS];
    int64_t s = 0;
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
        v[k] = (i < n) ? in[i] : 0;
        s += v[k];
    }
    int64_t run = sums[blockIdx.x] + block_exclusive_scan<int64_t>(s, &tot);
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
}

template <class T>
int scan_impl(gx_ctx *ctx, const T *in, T *out, int64_t n, T *total_host) {
    if (n <= 0) {
        if (total_host) *total_host = 0;
        return GX_OK;
    }
    int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    GX_TRY(gx_ensure(ctx, ctx->scratch_g, sizeof(T) * (nb + 1)));
    T *sums = dptr<T>(ctx->scratch_g);
    k_scan_sums<T><<<(unsigned)nb, SCAN_THREADS, 0, ctx->stream>>>(in, n, sums);
    k_scan_single<T><<<1, SCAN_THREADS, 0, ctx->stream>>>(sums, nb, sums + nb);
    k_scan_apply<T><<<(unsigned)nb, SCAN_THREADS, 0, ctx->stream>>>(in, out, n, sums);
    ctx->launches += 3;
    GX_CUDA(ctx, cudaGetLastError());
    if (total_host) {
        GX_CUDA(ctx, cudaMemcpyAsync(total_host, sums + nb, sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return GX_OK;
}

// ------------------------------------------------------------------ radix sort
constexpr int RS_WARPS = 8;
constexpr int RS_ROUNDS = 8;
constexpr int RS_WARP_ITEMS = 32 * RS_ROUNDS;          // 256
constexpr int RS_TILE = RS_WARPS * RS_WARP_ITEMS;      // 2048
constexpr int RS_BINS = 256;

__global__ void k_rs_hist(const uint64_t *keys, int64_t n, int shift, unsigned mask, unsigned *hist, int64_t nb) {
    __shared__ unsigned h[RS_BINS];
    for (int i = threadIdx.x; i < RS_BINS; i += blockDim.x) h[i] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * RS_TILE;
    for (int k = threadIdx.x; k < RS_TILE; k += blockDim.x) {
        int64_t i = base + k;
        if (i < n) atomicAdd(&h[(unsigned)(keys[i] >> shift) & mask], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RS_BINS; d += blockDim.x) hist[(int64_t)d * nb + blockIdx.x] = h[d];
}

// flag = 1 if every key has the same digit (the pass copies instead of scattering)
__global__ void k_rs_uniform(const unsigned *offs, int64_t nb, int64_t n, unsigned *flag) {
    int d = threadIdx.x;
    if (d >= RS_BINS) return;
    int64_t lo = offs[(int64_t)d * nb];
    int64_t hi = (d + 1 < RS_BINS) ? (int64_t)offs[(int64_t)(d + 1) * nb] : n;
    if (hi - lo == n) *flag = 1u;
}

__global__ void __launch_bounds__(RS_WARPS * 32) k_rs_scatter(const uint64_t *kin, const uint32_t *vin,
                                                             uint64_t *kout, uint32_t *vout, int64_t n,
                                                             int shift, unsigned mask, const unsigned *offs,
                                                             int64_t nb, const unsigned *uniform) {
    if (*uniform) {  // every key has the same digit: the stable order is the present one
        for (int64_t i = (int64_t)blockIdx.x * RS_TILE + threadIdx.x; i < n && i < (int64_t)(blockIdx.x + 1) * RS_TILE;
             i += blockDim.x) {
            kout[i] = kin[i];
            vout[i] = vin[i];
        }
        return;
    }
    __shared__ unsigned cnt[RS_WARPS][RS_BINS];
    for (int i = threadIdx.x; i < RS_WARPS * RS_BINS; i += blockDim.x) (&cnt[0][0])[i] = 0;
    __syncthreads();
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned lt = (1u << lane) - 1u;
    int64_t base = (int64_t)blockIdx.x * RS_TILE + (int64_t)w * RS_WARP_ITEMS;
    uint64_t k[RS_ROUNDS];
    uint32_t v[RS_ROUNDS];
    unsigned d[RS_ROUNDS], rk[RS_ROUNDS];
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        int64_t i = base + r * 32 + lane;
        bool ok = i < n;
        k[r] = ok ? kin[i] : 0ull;
        v[r] = ok ? vin[i] : 0u;
        d[r] = ok ? ((unsigned)(k[r] >> shift) & mask) : 0xFFFFFFFFu;
        unsigned peers = __match_any_sync(0xffffffffu, d[r]);
        int leader = __ffs(peers) - 1;
        unsigned c = ok ? cnt[w][d[r]] : 0u;
        __syncwarp();
        if (ok && lane == leader) cnt[w][d[r]] = c + __popc(peers);
        __syncwarp();
        rk[r] = c + __popc(peers & lt);
    }
    __syncthreads();
    for (int dd = threadIdx.x; dd < RS_BINS; dd += blockDim.x) {
        unsigned run = 0;
        for (int ww = 0; ww < RS_WARPS; ww++) {
            unsigned t = cnt[ww][dd];
            cnt[ww][dd] = run;
            run += t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        if (d[r] == 0xFFFFFFFFu) continue;
        int64_t pos = (int64_t)offs[(int64_t)d[r] * nb + blockIdx.x] + cnt[w][d[r]] + rk[r];
        kout[pos] = k[r];
        vout[pos] = v[r];
    }
}

}  // namespace

int gx_exclusive_scan_i64(gx_ctx *ctx, const int64_t *in, int64_t *out, int64_t n) {
    return scan_impl<int64_t>(ctx, in, out, n, nullptr);
}

int gx_exclusive_scan_i64_devn(gx_ctx *ctx, const int64_t *in, int64_t *out, const int64_t *n_dev, int64_t n_add,
                               int64_t n_cap, int64_t *total_dev) {
    return gx_exclusive_scan_i64_devn_multi(ctx, in, out, 1, 0, n_dev, n_add, n_cap, total_dev);
}

int gx_exclusive_scan_i64_devn_multi(gx_ctx *ctx, const int64_t *in, int64_t *out, int m, int64_t stride,
                                     const int64_t *n_dev, int64_t n_add, int64_t n_cap, int64_t *total_dev) {
    if (n_cap <= 0 || m <= 0) return GX_OK;
    int64_t nb = (n_cap + SCAN_TILE - 1) / SCAN_TILE;
    GX_TRY(gx_ensure(ctx, ctx->scratch_g, sizeof(int64_t) * (size_t)m * (nb + 1)));
    int64_t *sums = dptr<int64_t>(ctx->scratch_g);
    const dim3 grid((unsigned)nb, (unsigned)m);
    k_scan_sums_dn<<<grid, SCAN_THREADS, 0, ctx->stream>>>(in, n_dev, n_add, n_cap, sums, stride);
    k_scan_single_dn<<<(unsigned)m, SCAN_THREADS, 0, ctx->stream>>>(sums, nb, total_dev);
    k_scan_apply_dn<<<grid, SCAN_THREADS, 0, ctx->stream>>>(in, out, n_dev, n_add, n_cap, sums, stride);
    ctx->launches += 3;
    GX_CUDA(ctx, cudaGetLastError());
    return GX_OK;
}

int gx_exclusive_scan_i32(gx_ctx *ctx, const int32_t *in, int32_t *out, int64_t n, int32_t *total_host) {
    return scan_impl<int32_t>(ctx, in, out, n, total_host);
}

// Stable sort of (keys, vals) by key bits [begin_bit, end_bit).  Ping-pongs with the
// *_alt buffers; *result_in_alt tells where the sorted data ended up.
int gx_radix_sort_u64(gx_ctx *ctx, uint64_t *keys, uint32_t *vals, int64_t n, int begin_bit, int end_bit,
                      uint64_t *keys_alt, uint32_t *vals_alt, bool *result_in_alt) {
    *result_in_alt = false;
    if (n <= 1) return GX_OK;
    int64_t nb = (n + RS_TILE - 1) / RS_TILE;
    if (nb * RS_BINS > 0x7fffffffLL) return gx_fail(ctx, GX_ERR_CAP_EXCEEDED, "radix sort: too many items");
    GX_TRY(gx_ensure(ctx, ctx->scratch_e, sizeof(unsigned) * (size_t)(nb * RS_BINS + 1)));
    GX_TRY(gx_ensure(ctx, ctx->scratch_f, sizeof(unsigned) * 4));
    unsigned *hist = dptr<unsigned>(ctx->scratch_e);
    unsigned *flag = dptr<unsigned>(ctx->scratch_f);
    uint64_t *ki = keys, *ko = keys_alt;
    uint32_t *vi = vals, *vo = vals_alt;
    for (int shift = begin_bit; shift < end_bit; shift += 8) {
        int bits = end_bit - shift < 8 ? end_bit - shift : 8;
        unsigned mask = (1u << bits) - 1u;
        k_rs_hist<<<(unsigned)nb, 256, 0, ctx->stream>>>(ki, n, shift, mask, hist, nb);
        ctx->launches++;
        int32_t total = 0;
        GX_TRY(scan_impl<int32_t>(ctx, reinterpret_cast<int32_t *>(hist), reinterpret_cast<int32_t *>(hist),
                                  nb * RS_BINS, nullptr));
        GX_CUDA(ctx, cudaMemsetAsync(flag, 0, sizeof(unsigned), ctx->stream));
        k_rs_uniform<<<1, RS_BINS, 0, ctx->stream>>>(hist, nb, n, flag);
        ctx->launches++;
        (void)total;
        // the uniform-digit case is decided on the device (a copy instead of the scatter),
        // so the passes run without a host round trip
        k_rs_scatter<<<(unsigned)nb, RS_WARPS * 32, 0, ctx->stream>>>(ki, vi, ko, vo, n, shift, mask, hist, nb, flag);
        ctx->launches++;
        GX_CUDA(ctx, cudaGetLastError());
        uint64_t *tk = ki; ki = ko; ko = tk;
        uint32_t *tv = vi; vi = vo; vo = tv;
    }
    *result_in_alt = (ki == keys_alt);
    return GX_OK;
}
