// gx_fmm.cu -- order dispatch of the force passes (kernels in gx_fmm_impl.cuh,
// instantiated per order in gx_fmm_p*.cu so they compile in parallel) and the
// host-built derivative polynomial table of the REF mode.
#include "gx_internal.cuh"

int gx_run_forces_0(gx_ctx *ctx, bool timed);
int gx_run_forces_1(gx_ctx *ctx, bool timed);
int gx_run_forces_2(gx_ctx *ctx, bool timed);
int gx_run_forces_3(gx_ctx *ctx, bool timed);
int gx_run_forces_4(gx_ctx *ctx, bool timed);
int gx_run_forces_5(gx_ctx *ctx, bool timed);
int gx_run_forces_6(gx_ctx *ctx, bool timed);
int gx_run_forces_7(gx_ctx *ctx, bool timed);
int gx_run_forces_8(gx_ctx *ctx, bool timed);
int gx_run_forces_9(gx_ctx *ctx, bool timed);
int gx_run_forces_10(gx_ctx *ctx, bool timed);
int gx_run_forces_11(gx_ctx *ctx, bool timed);
int gx_run_forces_12(gx_ctx *ctx, bool timed);
int gx_run_forces_13(gx_ctx *ctx, bool timed);
int gx_run_forces_14(gx_ctx *ctx, bool timed);
int gx_run_forces_15(gx_ctx *ctx, bool timed);
int gx_run_forces_16(gx_ctx *ctx, bool timed);

// Polynomial numerators N_{k,l}(x, y; eps^2) of compute_kernel_derivs
// (lib.rs:1059-1130), built by the reference's recurrence, as a dense table
// poly[(k*S + l)*S*S + a*S + b], S = 2p+1.
int gx_poly_table_host(int p, double eps, std::vector<double> &out) {
    int order = 2 * p, S = order + 1;
    out.assign((size_t)S * S * S * S, 0.0);
    double eps2 = eps * eps;
    auto PL = [&](int k, int l) { return out.data() + ((size_t)k * S + l) * S * S; };
    PL(0, 0)[0] = -1.0;
    for (int n = 1; n <= order; n++)
        for (int k = 0; k <= n; k++) {
            int l = n - k;
            double *coeff = PL(k, l);
            if (k > 0) {
                const double *prev = PL(k - 1, l);
                int mm = 1 + 2 * (k - 1) + 2 * l;
                for (int a = 0; a < S; a++)
                    for (int b = 0; b < S - a; b++) {
                        double c = prev[a * S + b];
                        if (c == 0.0) continue;
                        if (a > 0) {
                            double dc = c * (double)a;
                            if (a + 1 < S) coeff[(a + 1) * S + b] += dc;
                            if (b + 2 < S) coeff[(a - 1) * S + b + 2] += dc;
                            coeff[(a - 1) * S + b] += dc * eps2;
                        }
                    }
                for (int a = 0; a < S; a++)
                    for (int b = 0; b < S - a; b++) {
                        double c = prev[a * S + b];
                        if (c == 0.0) continue;
                        if (a + 1 < S) coeff[(a + 1) * S + b] -= (double)mm * c;
                    }
            } else if (l > 0) {
                const double *prev = PL(k, l - 1);
                int mm = 1 + 2 * k + 2 * (l - 1);
                for (int a = 0; a < S; a++)
                    for (int b = 0; b < S - a; b++) {
                        double c = prev[a * S + b];
                        if (c == 0.0) continue;
                        if (b > 0) {
                            double dc = c * (double)b;
                            if (a + 2 < S) coeff[(a + 2) * S + b - 1] += dc;
                            if (b + 1 < S) coeff[a * S + b + 1] += dc;
                            coeff[a * S + b - 1] += dc * eps2;
                        }
                    }
                for (int a = 0; a < S; a++)
                    for (int b = 0; b < S - a; b++) {
                        double c = prev[a * S + b];
                        if (c == 0.0) continue;
                        if (b + 1 < S) coeff[a * S + b + 1] -= (double)mm * c;
                    }
            }
        }
    return GX_OK;
}

int gx_forces_device(gx_ctx *ctx, bool timed) {
    switch (ctx->p) {
#define GX_CASE(PP) \
    case PP: return gx_run_forces_##PP(ctx, timed);
        GX_CASE(0) GX_CASE(1) GX_CASE(2) GX_CASE(3) GX_CASE(4) GX_CASE(5) GX_CASE(6) GX_CASE(7) GX_CASE(8)
        GX_CASE(9) GX_CASE(10) GX_CASE(11) GX_CASE(12) GX_CASE(13) GX_CASE(14) GX_CASE(15) GX_CASE(16)
#undef GX_CASE
        default:
            return gx_fail(ctx, GX_ERR_INVALID_ARG, "p must be in 0..16");
    }
}
