// gx_kdk.cu -- device-resident leapfrog, diagnostics and the sampled exact sum.
//
//  * leapfrog_kdk (galax-integrate/src/lib.rs:158-189): kick dt/2, drift dt,
//    force (static tree), kick dt/2 -- FP64 state, separately rounded mul/add;
//  * diagnostics (galax-core/src/lib.rs:1638-1683): KE, FMM PE, momentum, Lz as
//    deterministic two-stage block reductions (fixed grid, fixed tree order);
//  * validate_fmm's exact sum (lib.rs:1537-1553) for sampled targets.
#include <mutex>

#include "gx_internal.cuh"

namespace {

constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 304;  // 2 x 152 SMs

__global__ void k_kick_drift(int64_t n, double h, double dt, double *x, double *y, double *vx, double *vy,
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

__global__ void k_kick(int64_t n, double h, double *vx, double *vy, const double *ax, const double *ay) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vx[i] = __dadd_rn(vx[i], __dmul_rn(ax[i], h));
    vy[i] = __dadd_rn(vy[i], __dmul_rn(ay[i], h));
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) r += sh[k];
    __syncthreads();
    return r;
}

// per block: {KE, PE, px, py, Lz} over a grid-stride range
__global__ void k_diag_partial(int64_t n, const double *x, const double *y, const double *vx, const double *vy,
                               const double *m, const double *ax, const double *ay, double *part) {
    __shared__ double sh[RED_THREADS / 32];
    double ke = 0, pe = 0, px = 0, py = 0, lz = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double mi = m[i], u = vx[i], v = vy[i], xi = x[i], yi = y[i];
        double v2 = __dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v));
        ke += __dmul_rn(__dmul_rn(0.5, mi), v2);
        double am = sqrt(__dadd_rn(__dmul_rn(ax[i], ax[i]), __dmul_rn(ay[i], ay[i])));
        double r = fmax(sqrt(__dadd_rn(__dmul_rn(xi, xi), __dmul_rn(yi, yi))), 1.0);
        pe += __dmul_rn(__dmul_rn(mi, am), r);
        px += __dmul_rn(mi, u);
        py += __dmul_rn(mi, v);
        lz += __dmul_rn(mi, __dsub_rn(__dmul_rn(xi, v), __dmul_rn(yi, u)));
    }
    double s[5] = {ke, pe, px, py, lz};
    for (int k = 0; k < 5; k++) {
        double t = block_sum(s[k], sh);
        if (threadIdx.x == 0) part[k * gridDim.x + blockIdx.x] = t;
    }
}

__global__ void k_diag_final(const double *part, int nb, double *out) {
    __shared__ double sh[RED_THREADS / 32];
    for (int k = 0; k < 5; k++) {
        double v = 0.0;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) v += part[k * nb + b];
        double t = block_sum(v, sh);
        if (threadIdx.x == 0) out[k] = (k == 1) ? -0.5 * t : t;
    }
}

// one block per sampled target
__global__ void k_n2_sampled(int64_t n, const double *x, const double *y, const double *m, double eps2,
                             const int64_t *idx, double *ax, double *ay) {
    __shared__ double sh[RED_THREADS / 32];
    int64_t i = idx[blockIdx.x];
    double xi = x[i], yi = y[i];
    double fx = 0.0, fy = 0.0;
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        if (j == i) continue;
        double dx = x[j] - xi, dy = y[j] - yi;
        double r2 = dx * dx + dy * dy + eps2;
        double ir = 1.0 / sqrt(r2);
        double f = m[j] * (ir * (ir * ir));
        fx += f * dx;
        fy += f * dy;
    }
    double tx = block_sum(fx, sh);
    double ty = block_sum(fy, sh);
    if (threadIdx.x == 0) {
        ax[blockIdx.x] = tx;
        ay[blockIdx.x] = ty;
    }
}

}  // namespace

int gx_diag_device(gx_ctx *ctx, double out[5]) {
    GX_TRY(gx_ensure(ctx, ctx->red, sizeof(double) * (5 * RED_BLOCKS + 8)));
    double *part = dptr<double>(ctx->red), *res = part + 5 * RED_BLOCKS;
    int64_t n = ctx->n_bodies;
    k_diag_partial<<<RED_BLOCKS, RED_THREADS, 0, ctx->stream>>>(n, dptr<double>(ctx->x), dptr<double>(ctx->y),
                                                                dptr<double>(ctx->vx), dptr<double>(ctx->vy),
                                                                dptr<double>(ctx->m), dptr<double>(ctx->ax),
                                                                dptr<double>(ctx->ay), part);
    k_diag_final<<<1, RED_THREADS, 0, ctx->stream>>>(part, RED_BLOCKS, res);
    ctx->launches += 2;
    GX_CUDA(ctx, cudaGetLastError());
    GX_CUDA(ctx, cudaMemcpyAsync(out, res, sizeof(double) * 5, cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GX_OK;
}

int gx_kdk_device(gx_ctx *ctx, int64_t n_steps, double dt, int64_t energy_every, double *diag, int64_t *n_diag,
                  int64_t rebuild_every) {
    int64_t n = ctx->n_bodies, nd = 0;
    double h = 0.5 * dt;
    for (int64_t step = 0; step < n_steps; step++) {
        k_kick_drift<<<gx_blocks(n, 256), 256, 0, ctx->stream>>>(n, h, dt, dptr<double>(ctx->x), dptr<double>(ctx->y),
                                                                 dptr<double>(ctx->vx), dptr<double>(ctx->vy),
                                                                 dptr<double>(ctx->ax), dptr<double>(ctx->ay));
        ctx->launches++;
        if (rebuild_every > 0 && (step + 1) % rebuild_every == 0) {
            // the tree of the drifted positions (the bodies, ids and accelerations are permuted with it)
            GX_TRY(gx_rebuild_internal(ctx));
            GX_TRY(gx_ensure_plan_public(ctx));
        }
        GX_TRY(gx_forces_device(ctx, false));
        k_kick<<<gx_blocks(n, 256), 256, 0, ctx->stream>>>(n, h, dptr<double>(ctx->vx), dptr<double>(ctx->vy),
                                                           dptr<double>(ctx->ax), dptr<double>(ctx->ay));
        ctx->launches++;
        GX_CUDA(ctx, cudaGetLastError());
        if (energy_every > 0 && (step + 1) % energy_every == 0) {
            double d[5];
            GX_TRY(gx_diag_device(ctx, d));
            if (diag) {
                double *row = diag + 6 * nd;
                row[0] = (double)(step + 1);
                row[1] = d[0];
                row[2] = d[1];
                row[3] = d[2];
                row[4] = d[3];
                row[5] = d[4];
            }
            nd++;
        }
    }
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (n_diag) *n_diag = nd;
    return GX_OK;
}

int gx_n2_device(gx_ctx *ctx, const int64_t *idx, int64_t n_idx, double *ax, double *ay) {
    if (n_idx <= 0) return GX_OK;
    GX_TRY(gx_ensure(ctx, ctx->scratch_a, sizeof(int64_t) * (size_t)n_idx + sizeof(double) * 2 * (size_t)n_idx));
    int64_t *didx = dptr<int64_t>(ctx->scratch_a);
    double *dax = reinterpret_cast<double *>(didx + n_idx), *day = dax + n_idx;
    for (int64_t k = 0; k < n_idx; k++)
        if (idx[k] < 0 || idx[k] >= ctx->n_bodies) return gx_fail(ctx, GX_ERR_INVALID_ARG, "n2: index out of range");
    GX_CUDA(ctx, cudaMemcpyAsync(didx, idx, sizeof(int64_t) * n_idx, cudaMemcpyHostToDevice, ctx->stream));
    k_n2_sampled<<<(unsigned)n_idx, RED_THREADS, 0, ctx->stream>>>(ctx->n_bodies, dptr<double>(ctx->x),
                                                                   dptr<double>(ctx->y), dptr<double>(ctx->m),
                                                                   ctx->eps * ctx->eps, didx, dax, day);
    ctx->launches++;
    GX_CUDA(ctx, cudaGetLastError());
    GX_CUDA(ctx, cudaMemcpyAsync(ax, dax, sizeof(double) * n_idx, cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaMemcpyAsync(ay, day, sizeof(double) * n_idx, cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GX_OK;
}

// ---------------------------------------------------------------- allocation-free variant
// gx_n2_sampled_static: the sampled exact sum without a context and without any
// device allocation.  Some callers cannot allocate device memory at the moment
// they want a force check: a simulation whose device memory is owned by another
// runtime's caching allocator (which may already hold nearly all of HBM, so a
// cudaMalloc would fail or fragment it).  Their device arrays are passed in; the
// per-sample indices and results are staged through the file-scope array below
// instead of context scratch.  The call copies through pageable host memory and
// synchronises its stream, so that stream must not be capturing.
//
// The array is GX_N2_STATIC_MAX_SAMPLES * 24 bytes (96 KiB); every GPU that loads
// this library holds it until the process exits.  All calls on a device share it
// and it keeps the last call's contents: each call overwrites every slot it reads
// (indices, then one result per sample), so nothing has to start at zero, but
// calls that overlap on the GPU (other streams, other host threads) race on it.
namespace {
static __device__ __align__(256) unsigned char g_n2_static_scratch[GX_N2_STATIC_MAX_SAMPLES *
                                                                   (sizeof(int64_t) + 2 * sizeof(double))];
// Device address of the array per device ordinal, found once per device with that
// device current (the host-side symbol is a stand-in, not a device address) and kept
// for the life of the process: it belongs to the device's primary context, so a
// caller's cudaDeviceReset ends the use of this entry point in that process.
constexpr int kMaxDevices = 64;
void *g_n2_static_addr[kMaxDevices] = {};
std::mutex g_n2_static_mu;
}  // namespace

extern "C" int gx_n2_sampled_static(const double *x, const double *y, const double *m, int64_t n, double eps,
                                    const int64_t *idx, int64_t n_idx, double *ax, double *ay, void *stream) {
    if (n < 0 || n_idx < 0 || !(eps >= 0.0)) return GX_ERR_INVALID_ARG;
    if (n_idx > GX_N2_STATIC_MAX_SAMPLES) return GX_ERR_CAP_EXCEEDED;
    if (n_idx == 0) return GX_OK;
    if (!x || !y || !m || !idx || !ax || !ay) return GX_ERR_INVALID_ARG;
    for (int64_t k = 0; k < n_idx; k++)
        if (idx[k] < 0 || idx[k] >= n) return GX_ERR_INVALID_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GX_ERR_INIT;
    void *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_n2_static_mu);
        if (!g_n2_static_addr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_n2_static_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return GX_ERR_KERNEL_LOAD;
            }
            g_n2_static_addr[dev] = p;
        }
        base = g_n2_static_addr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int64_t *didx = static_cast<int64_t *>(base);
    double *dax = reinterpret_cast<double *>(didx + GX_N2_STATIC_MAX_SAMPLES);
    double *day = dax + GX_N2_STATIC_MAX_SAMPLES;
    if (cudaMemcpyAsync(didx, idx, sizeof(int64_t) * n_idx, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        cudaGetLastError();
        return GX_ERR_CUDA;
    }
    k_n2_sampled<<<(unsigned)n_idx, RED_THREADS, 0, st>>>(n, x, y, m, eps * eps, didx, dax, day);
    if (cudaGetLastError() != cudaSuccess) return GX_ERR_CUDA;
    if (cudaMemcpyAsync(ax, dax, sizeof(double) * n_idx, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(ay, day, sizeof(double) * n_idx, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return GX_ERR_CUDA;
    }
    return GX_OK;
}
