// gx_lists.cu -- device interaction lists and static per-tree plans.
//
//  * V-list: InteractionLists::build (galax-core/src/lib.rs:947-1025)
//  * U-list: build_p2p_lists (lib.rs:1358-1392)
//  * build_constrained's neighbour search (neighbors_geometric, lib.rs:382-423)
//  * REF P2P gather lists: p2p (lib.rs:1395-1462) updates both sides of a leaf
//    pair when the partner id is higher and skips lower partners, so leaf a
//    receives from b != a iff (b > a and b in U(a)) or (b < a and a in U(b)).
//  * REF M2L derivative plan: m2l's cache (lib.rs:1209-1247) keyed on
//    (dx as i64, dy as i64) where the first pair in (target id, slot) order wins.
//  * ACCURATE mode near/far lists (not in the reference).
//
// The reference scans every node of a level for every query.  Here each query
// walks a bounding-volume hierarchy built over the level's nodes in id order
// (buckets of 8 consecutive ids), visiting buckets left to right, so candidates
// come out in ascending id order; the reference's own floating-point test is
// then applied to each candidate, so the lists are identical.  Boxes are widened
// by a margin that covers every rounding of the exact test.  Levels that hold a
// node with a non-finite box fall back to scanning the level in id order.
#include <climits>

#include <algorithm>
#include <set>

#include "gx_internal.cuh"

int gx_tree_rebuild_with_splits(gx_ctx *ctx, int64_t n_max, const double bounds[4], const std::vector<int64_t> &splits);
int gx_add_offsets(gx_ctx *ctx, const int64_t *o, int64_t *dst, int64_t c, int64_t add);

namespace {

constexpr int BVH_B = 8;

struct Level {
    int64_t s, e, p2;
    double4 *box;
    bool brute;
    double maxabs;
    double4 *cbox;  // optional: per BVH node, bounding box of the children's centres
    double *cmh;    //           and the minimum child half-width (-inf if any child is non-finite)
    double cmax;
};

__device__ __forceinline__ bool finite3(double a, double b, double c) {
    return isfinite(a) && isfinite(b) && isfinite(c);
}

__device__ __forceinline__ void atomic_max_pos(double *addr, double v) {
    // non-negative doubles order like their bit patterns
    atomicMax(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

__global__ void k_bvh_leaves(int64_t s, int64_t cnt, int64_t p2, const double *cx, const double *cy, const double *hw,
                             double4 *box, unsigned *nonfinite, double *maxabs) {
    int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p2) return;
    double4 bx = make_double4(INFINITY, -INFINITY, INFINITY, -INFINITY);
    double ma = 0.0;
    unsigned nf = 0;
    for (int64_t k = b * BVH_B; k < b * BVH_B + BVH_B && k < cnt; k++) {
        int64_t id = s + k;
        double c_x = cx[id], c_y = cy[id], h = hw[id];
        if (!finite3(c_x, c_y, h)) { nf++; continue; }
        bx.x = fmin(bx.x, c_x - h); bx.y = fmax(bx.y, c_x + h);
        bx.z = fmin(bx.z, c_y - h); bx.w = fmax(bx.w, c_y + h);
        ma = fmax(ma, fabs(c_x) + fabs(c_y) + fabs(h));
    }
    box[p2 + b] = bx;
    if (nf) atomicAdd(nonfinite, nf);
    if (ma > 0.0) atomic_max_pos(maxabs, ma);
}

__global__ void k_bvh_up(int64_t lo, int64_t hi, double4 *box) {
    int64_t h = lo + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= hi) return;
    double4 a = box[2 * h], b = box[2 * h + 1];
    box[h] = make_double4(fmin(a.x, b.x), fmax(a.y, b.y), fmin(a.z, b.z), fmax(a.w, b.w));
}

// Calls f(id) for every node of the level whose box may overlap the query box,
// in ascending id order.  Returns false if the traversal stack overflowed.
template <class F>
__device__ bool level_query(const Level &L, const double *cx, const double *cy, const double *hw, double qx0,
                            double qx1, double qy0, double qy1, bool qfinite, F &&f) {
    if (L.brute || !qfinite) {
        for (int64_t id = L.s; id < L.e; id++) f(id);
        return true;
    }
    int64_t stack[64];
    int sp = 0;
    stack[sp++] = 1;
    while (sp > 0) {
        int64_t h = stack[--sp];
        double4 b = L.box[h];
        if (b.x > qx1 || b.y < qx0 || b.z > qy1 || b.w < qy0) continue;
        if (h >= L.p2) {
            int64_t k0 = (h - L.p2) * BVH_B;
            for (int64_t k = k0; k < k0 + BVH_B && L.s + k < L.e; k++) {
                int64_t id = L.s + k;
                double c_x = cx[id], c_y = cy[id], hh = hw[id];
                if (c_x - hh > qx1 || c_x + hh < qx0 || c_y - hh > qy1 || c_y + hh < qy0) continue;
                f(id);
            }
        } else {
            if (sp + 2 > 64) return false;
            stack[sp++] = 2 * h + 1;
            stack[sp++] = 2 * h;
        }
    }
    return true;
}

__device__ __forceinline__ double margin(const Level &L, double qabs) { return 1e-15 + 1e-12 * (L.maxabs + qabs + 1.0); }

// V-list parent test (lib.rs:990-995): pn skipped iff dx > h_sum + 1e-15 || dy > h_sum + 1e-15
__device__ __forceinline__ bool vparent_near(const double *cx, const double *cy, const double *hw, int64_t P, int64_t pn) {
    double dx = fabs(__dsub_rn(cx[pn], cx[P])), dy = fabs(__dsub_rn(cy[pn], cy[P]));
    double hs = __dadd_rn(hw[P], hw[pn]);
    double lim = __dadd_rn(hs, 1e-15);
    return !(dx > lim || dy > lim);
}

// V-list child adjacency (lib.rs:1000-1006)
__device__ __forceinline__ bool vchild_adjacent(const double *cx, const double *cy, const double *hw, int64_t n, int64_t c) {
    double cdx = fabs(__dsub_rn(cx[c], cx[n])), cdy = fabs(__dsub_rn(cy[c], cy[n]));
    double lim = __dadd_rn(__dadd_rn(hw[n], hw[c]), 1e-15);
    return (cdx <= lim) && (cdy <= lim);
}

// U-list touch (lib.rs:1380-1384)
__device__ __forceinline__ bool utouch(const double *cx, const double *cy, const double *hw, int64_t a, int64_t b) {
    double dx = fabs(__dsub_rn(cx[a], cx[b])), dy = fabs(__dsub_rn(cy[a], cy[b]));
    double lim = __dadd_rn(__dadd_rn(hw[a], hw[b]), 1e-15);
    return dx <= lim && dy <= lim;
}

__device__ __forceinline__ void qbox(const double *cx, const double *cy, const double *hw, int64_t q, const Level &L,
                                     double &x0, double &x1, double &y0, double &y1, bool &fin) {
    double c_x = cx[q], c_y = cy[q], h = hw[q];
    fin = finite3(c_x, c_y, h);
    double mg = margin(L, fabs(c_x) + fabs(c_y) + fabs(h));
    x0 = c_x - h - mg; x1 = c_x + h + mg; y0 = c_y - h - mg; y1 = c_y + h + mg;
}

__global__ void k_cenv_leaves(int64_t s, int64_t cnt, int64_t p2, const int4 *child, const double *cx,
                              const double *cy, const double *hw, double4 *cbox, double *cmh, double *cmax) {
    int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p2) return;
    double4 bx = make_double4(INFINITY, -INFINITY, INFINITY, -INFINITY);
    double mh = INFINITY, ma = 0.0;
    for (int64_t k = b * BVH_B; k < b * BVH_B + BVH_B && k < cnt; k++) {
        int4 c4 = child[s + k];
        int cc[4] = {c4.x, c4.y, c4.z, c4.w};
        for (int q = 0; q < 4; q++) {
            int c = cc[q];
            if (c < 0) continue;
            double c_x = cx[c], c_y = cy[c], h = hw[c];
            if (!finite3(c_x, c_y, h)) { mh = -INFINITY; continue; }
            bx.x = fmin(bx.x, c_x); bx.y = fmax(bx.y, c_x);
            bx.z = fmin(bx.z, c_y); bx.w = fmax(bx.w, c_y);
            mh = fmin(mh, h);
            ma = fmax(ma, fabs(c_x) + fabs(c_y) + h);
        }
    }
    cbox[p2 + b] = bx;
    cmh[p2 + b] = mh;
    if (ma > 0.0) atomic_max_pos(cmax, ma);
}

__global__ void k_cenv_up(int64_t lo, int64_t hi, double4 *cbox, double *cmh) {
    int64_t h = lo + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= hi) return;
    double4 a = cbox[2 * h], b = cbox[2 * h + 1];
    cbox[h] = make_double4(fmin(a.x, b.x), fmax(a.y, b.y), fmin(a.z, b.z), fmax(a.w, b.w));
    cmh[h] = fmin(cmh[2 * h], cmh[2 * h + 1]);
}

// V-list of every node of level lv, one thread per node: walks the parent level's
// hierarchy in ascending id order, pruning subtrees with no parent near P and
// subtrees whose every child is certainly adjacent to the node; stops at the cap.
__global__ void k_vlist_node(int64_t s0, int64_t e0, Level pl, const int32_t *parent, const int4 *child,
                             const double *cx, const double *cy, const double *hw, uint32_t *vdata, uint8_t *vlen,
                             unsigned *status) {
    int64_t n = s0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= e0) return;
    int32_t P = parent[n];
    int len = 0;
    auto visit = [&](int64_t pn) {
        if (pn == P || !vparent_near(cx, cy, hw, P, pn)) return;
        int4 c4 = child[pn];
        int cc[4] = {c4.x, c4.y, c4.z, c4.w};
        for (int k = 0; k < 4; k++) {
            int c = cc[k];
            if (c < 0 || vchild_adjacent(cx, cy, hw, n, c)) continue;
            if (len < GX_LIST_CAP) vdata[n * GX_LIST_CAP + len++] = (uint32_t)c;
        }
    };
    if (P >= 0) {
        if (pl.brute) {
            for (int64_t pn = pl.s; pn < pl.e && len < GX_LIST_CAP; pn++) visit(pn);
        } else {
            double pcx = cx[P], pcy = cy[P], phw = hw[P];
            bool pfin = finite3(pcx, pcy, phw);
            double mg = margin(pl, fabs(pcx) + fabs(pcy) + fabs(phw));
            double qx0 = pcx - phw - mg, qx1 = pcx + phw + mg, qy0 = pcy - phw - mg, qy1 = pcy + phw + mg;
            double ncx = cx[n], ncy = cy[n], nhw = hw[n];
            double dl = 1e-12 * (fabs(ncx) + fabs(ncy) + fabs(nhw) + pl.cmax + 1.0);
            int64_t stack[64];
            int sp = 0;
            stack[sp++] = 1;
            while (sp > 0 && len < GX_LIST_CAP) {
                int64_t h = stack[--sp];
                double4 b = pl.box[h];
                if (pfin && (b.x > qx1 || b.y < qx0 || b.z > qy1 || b.w < qy0)) continue;
                double4 cbx = pl.cbox[h];
                double wx = fmax(fabs(cbx.x - ncx), fabs(cbx.y - ncx));
                double wy = fmax(fabs(cbx.z - ncy), fabs(cbx.w - ncy));
                double lim = nhw + pl.cmh[h] - dl;
                if (wx <= lim && wy <= lim) continue;  // every child adjacent to n
                if (h >= pl.p2) {
                    int64_t i0 = pl.s + (h - pl.p2) * BVH_B;
                    for (int64_t pn = i0; pn < i0 + BVH_B && pn < pl.e && len < GX_LIST_CAP; pn++) visit(pn);
                } else {
                    if (sp + 2 > 64) { atomicOr(status, GX_DEV_STACK_OVERFLOW); break; }
                    stack[sp++] = 2 * h + 1;
                    stack[sp++] = 2 * h;
                }
            }
        }
    }
    vlen[n] = (uint8_t)len;
}

__global__ void k_ulist(Level lv0, const double *cx, const double *cy, const double *hw, uint32_t *udata, uint8_t *ulen,
                        unsigned *status) {
    int64_t a = lv0.s + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= lv0.e) return;
    int len = 0;
    udata[a * GX_LIST_CAP + len++] = (uint32_t)a;
    double x0, x1, y0, y1;
    bool fin;
    qbox(cx, cy, hw, a, lv0, x0, x1, y0, y1, fin);
    bool ok = level_query(lv0, cx, cy, hw, x0, x1, y0, y1, fin, [&](int64_t b) {
        if (b == a || len >= GX_LIST_CAP) return;
        if (utouch(cx, cy, hw, a, b)) udata[a * GX_LIST_CAP + len++] = (uint32_t)b;
    });
    if (!ok) atomicOr(status, GX_DEV_STACK_OVERFLOW);
    ulen[a] = (uint8_t)len;
}

// REF P2P gather lists (the ownership rule of p2p, lib.rs:1395-1462): per receiving
// leaf a, {a} then ascending b with (b > a and b in U(a)) or (b < a and a in U(b)).
// Built by inverting the U-lists instead of searching geometry: every entry y of U(x)
// with y > x gives the pairs (receiver x, source y) and (receiver y, source x); a sort
// of the (receiver, source) keys orders each receiver's sources ascending.
__global__ void k_gather_count(int64_t nl, const uint32_t *udata, const uint8_t *ulen, int64_t *cnt) {
    int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nl) return;
    int64_t c = 0;
    for (int k = 1; k < ulen[x]; k++)
        if ((int64_t)udata[x * GX_LIST_CAP + k] > x) c += 2;
    cnt[x] = c;
}

__global__ void k_gather_emit(int64_t nl, const uint32_t *udata, const uint8_t *ulen, const int64_t *off,
                              uint64_t *keys) {
    int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nl) return;
    int64_t o = off[x];
    for (int k = 1; k < ulen[x]; k++) {
        uint64_t y = udata[x * GX_LIST_CAP + k];
        if ((int64_t)y > x) {
            keys[o++] = ((uint64_t)x << 32) | y;
            keys[o++] = (y << 32) | (uint64_t)x;
        }
    }
}

// per receiver: its range in the sorted keys (binary search) and list length 1 + range
__global__ void k_gather_ranges(int64_t nl, const uint64_t *keys, int64_t nk, int64_t *kstart, int64_t *len) {
    int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nl) return;
    auto lower = [&](uint64_t v) {
        int64_t lo = 0, hi = nk;
        while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if (keys[mid] < v) lo = mid + 1;
            else hi = mid;
        }
        return lo;
    };
    int64_t s = lower((uint64_t)a << 32), e = lower((uint64_t)(a + 1) << 32);
    kstart[a] = s;
    len[a] = 1 + (e - s);
}

__global__ void k_gather_fill(int64_t nl, const uint64_t *keys, const int64_t *kstart, const int64_t *off,
                              int32_t *out) {
    int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nl) return;
    int64_t o = off[a], n = off[a + 1] - o;
    out[o] = (int32_t)a;
    for (int64_t k = 1; k < n; k++) out[o + k] = (int32_t)(uint32_t)keys[kstart[a] + k - 1];
}

// Rust `f64 as i64`
__device__ __forceinline__ long long f64_as_i64(double v) {
    if (v != v) return 0;
    if (v >= 9223372036854775808.0) return LLONG_MAX;
    if (v < -9223372036854775808.0) return LLONG_MIN;
    return __double2ll_rz(v);
}

__global__ void k_ref_pair_keys(int64_t nn, const uint32_t *vdata, const uint8_t *vlen, const int64_t *voff,
                                const double *comx, const double *comy, uint64_t *klo, uint64_t *khi, uint32_t *pidx,
                                double *pdx, double *pdy) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t n = t / GX_LIST_CAP;
    int s = (int)(t % GX_LIST_CAP);
    if (n >= nn || s >= vlen[n]) return;
    uint32_t src = vdata[n * GX_LIST_CAP + s];
    double dx = __dsub_rn(comx[n], comx[src]), dy = __dsub_rn(comy[n], comy[src]);
    int64_t pi = voff[n] + s;
    klo[pi] = (uint64_t)f64_as_i64(dx);
    khi[pi] = (uint64_t)f64_as_i64(dy);
    pidx[pi] = (uint32_t)pi;
    pdx[pi] = dx;
    pdy[pi] = dy;
}

__global__ void k_gather_u64(const uint32_t *idx, const uint64_t *in, uint64_t *out, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[idx[i]];
}

__global__ void k_run_heads(const uint64_t *a, const uint64_t *b, int64_t n, int32_t *head) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    head[i] = (i == 0) ? 1 : (a[i] != a[i - 1] || b[i] != b[i - 1]);
}

__global__ void k_run_assign(const int32_t *head, const int32_t *hex, const uint32_t *pidx, int64_t n, int32_t *did,
                             int32_t *first_pair) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t k = hex[i] + head[i] - 1;
    did[pidx[i]] = k;
    if (head[i]) first_pair[k] = (int32_t)pidx[i];
}

// x^a by binary exponentiation: the expansion LLVM uses for f64::powi
__device__ __forceinline__ double powi_dev(double x, int a) {
    double r = 1.0;
    for (;;) {
        if (a & 1) r = __dmul_rn(r, x);
        a >>= 1;
        if (a == 0) break;
        x = __dmul_rn(x, x);
    }
    return r;
}

// compute_kernel_derivs (lib.rs:1040-1151) evaluated from the polynomial table
// (built on the host by the same recurrence): G^(k,l) = sum N_kl[a][b] x^a y^b / R^(1+2k+2l).
__global__ void k_ref_derivs(int64_t nk, const int32_t *first_pair, const double *pdx, const double *pdy,
                             const double *poly, int p, double eps, double *G) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    int S = 2 * p + 1;
    double x = pdx[first_pair[k]], y = pdy[first_pair[k]];
    double eps2 = __dmul_rn(eps, eps);
    double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), eps2);
    double r = __dsqrt_rn(r2);
    double inv_r[2 + 4 * GX_MAXP + 2];
    inv_r[1] = __ddiv_rn(1.0, r);
    for (int n = 3; n <= 1 + 2 * (2 * p); n += 2) inv_r[n] = __ddiv_rn(inv_r[n - 2], r2);
    double *g = G + k * (int64_t)S * S;
    for (int i = 0; i < S * S; i++) g[i] = 0.0;
    for (int kk = 0; kk < S; kk++)
        for (int l = 0; l < S - kk; l++) {
            const double *pl = poly + ((int64_t)kk * S + l) * S * S;
            double val = 0.0;
            for (int a = 0; a < S; a++)
                for (int b = 0; b < S - a; b++) {
                    double c = pl[a * S + b];
                    if (c != 0.0) val = __dadd_rn(val, __dmul_rn(__dmul_rn(c, powi_dev(x, a)), powi_dev(y, b)));
                }
            g[(kk + l) * S + l] = __dmul_rn(val, inv_r[1 + 2 * kk + 2 * l]);
        }
}

__global__ void k_u8_to_i64(const uint8_t *in, int64_t *out, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i];
}
// ---------------------------------------------------------------- accurate mode
// sqrt(dx*dx + dy*dy) with separately rounded operations: the same bits as the
// oracle, so near/far decisions agree exactly.
__device__ __forceinline__ double dist_rn(double dx, double dy) {
    return __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
}

// a warp per leaf, a lane per body: the maximum is exact in any order, and as the
// correctly rounded square root is monotone, the largest distance is the root of the
// largest squared distance (one FP64 square root per leaf instead of one per body)
__global__ void k_radius_leaves(int64_t nl, const double *x, const double *y, const double *comx, const double *comy,
                                const int32_t *bs, const int32_t *be, double *R) {
    const int64_t L = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (L >= nl) return;
    const double cx = comx[L], cy = comy[L];
    double r2 = 0.0;
    for (int32_t i = bs[L] + lane; i < be[L]; i += 32) {
        const double dx = x[i] - cx, dy = y[i] - cy;
        r2 = fmax(r2, __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r2 = fmax(r2, __shfl_xor_sync(0xffffffffu, r2, o));
    if (lane == 0) R[L] = __dsqrt_rn(r2);
}

__device__ __forceinline__ double radius_node(int64_t q, const int4 *child, const double *comx, const double *comy,
                                              const double *R) {
    const int4 c4 = child[q];
    const int cc[4] = {c4.x, c4.y, c4.z, c4.w};
    double r = 0.0;
    for (int k = 0; k < 4; k++) {
        const int c = cc[k];
        if (c < 0) continue;
        r = fmax(r, __dadd_rn(dist_rn(comx[c] - comx[q], comy[c] - comy[q]), R[c]));
    }
    return r;
}

__global__ void k_radius_parents(int64_t s, int64_t e, const int4 *child, const double *comx, const double *comy,
                                 double *R) {
    int64_t q = s + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= e) return;
    R[q] = radius_node(q, child, comx, comy, R);
}

// levels 1 .. L of single-child chains over the leaves (node x + l nl, child x + (l-1) nl):
// one thread walks each leaf's chain, the arithmetic of radius_node with one child.  The
// chain form is checked in the same plan attempt (k_chain_check), which is redone with
// per-level radii when it fails.
__global__ void k_radius_chain(int64_t nl, int L, const double *comx, const double *comy, double *R) {
    const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nl) return;
    double r = R[x];
    for (int l = 1; l <= L; l++) {
        const int64_t q = x + l * nl, c = q - nl;
        r = fmax(0.0, __dadd_rn(dist_rn(comx[c] - comx[q], comy[c] - comy[q]), r));
        R[q] = r;
    }
}

// the top levels (at most RADIUS_TOP nodes each) in one block, a barrier between levels
constexpr int RADIUS_TOP = 256;  // one SM's FP64 pipe: only the small levels
constexpr int RADIUS_TOP_THREADS = 256;
struct RadiusLevels {
    int64_t start[66];  // level_start of levels lo .. hi + 1
    int lo, hi;
};
__global__ void __launch_bounds__(RADIUS_TOP_THREADS) k_radius_top(RadiusLevels RL, const int4 *child,
                                                                   const double *comx, const double *comy, double *R) {
    for (int lv = RL.lo; lv <= RL.hi; lv++) {
        const int64_t s = RL.start[lv - RL.lo], e = RL.start[lv - RL.lo + 1];
        for (int64_t q = s + threadIdx.x; q < e; q += RADIUS_TOP_THREADS) R[q] = radius_node(q, child, comx, comy, R);
        __syncthreads();
    }
}

// Far when |com_a - com_b| theta > R_a + R_b, decided in FP32 and compared squared:
// the COM offset from the FP32 (hi, lo) split of each COM, the radii rounded to FP32
// once.  FP64 throughput on this part is a small fraction of FP32 and the plan tests
// ~10^8 pairs at 1M bodies; every operation is separately rounded so the oracle's
// decision is the same bit for bit.
__device__ __forceinline__ bool mac_far(const float4 *__restrict__ hl, const float *__restrict__ R32, int64_t a,
                                        int64_t b, float theta2) {
    const float4 A = hl[a], B = hl[b];
    const float ex = __fadd_rn(__fsub_rn(A.x, B.x), __fsub_rn(A.y, B.y));
    const float ey = __fadd_rn(__fsub_rn(A.z, B.z), __fsub_rn(A.w, B.w));
    const float d2 = __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey));
    const float s = __fadd_rn(R32[a], R32[b]);
    return __fmul_rn(d2, theta2) > __fmul_rn(s, s);
}

__global__ void k_to_f32(int64_t n, const double *in, float *out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)in[i];
}

// Per node x of a level: children of Near(parent(x)) split into far (M2L) and near,
// in the order (parent's near entry, child slot).  The parent's near list is cut into
// chunks of MAC_CHUNK entries and every (node, chunk) unit is one warp: the lanes take
// 32 consecutive entries at a time and place their children with a warp prefix sum.
// A wide leaf of the sparse halo can be near every other leaf; chunking spreads the
// nodes below it over many warps instead of one.
constexpr int MAC_CHUNK = 128;

// Plan counters on the device (the level loop runs without host round trips):
// running far / near list totals, the last level's near count, and overflow flags.
// Capacities are fixed for one attempt; a level that would exceed one sets its flag,
// every later kernel of the attempt returns at once, and the host grows the arrays
// and plans again.
enum { PC_FAR = 0, PC_NEAR = 1, PC_NEAR_LAST = 2, PC_OVF = 3, PC_N = 4 };
enum { OVF_UNITS = 1, OVF_FAR = 2, OVF_NEAR = 4, OVF_CHAIN = 8 };

__global__ void k_mac_nchunks(int64_t s, int64_t e, const int32_t *parent, const int32_t *near_cnt, int64_t *nch,
                              const int64_t *ctr) {
    if (ctr[PC_OVF]) return;
    int64_t x = s + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x > e) return;
    if (x == e) { nch[e - s] = 0; return; }
    int32_t P = parent[x];
    int64_t cand = P >= 0 ? near_cnt[P] : 0;
    nch[x - s] = (cand + MAC_CHUNK - 1) / MAC_CHUNK;
}

// unit -> (node, chunk) for the level's U = uoff[e - s] units; zero count slots at U
// so the count scans below end on the level totals
__global__ void k_mac_units(int64_t s, int64_t e, const int64_t *uoff, int64_t ucap, int32_t *unode, int32_t *uchunk,
                            int64_t *ufar, int64_t *unear, int64_t *ctr) {
    if (ctr[PC_OVF]) return;
    int64_t x = s + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= e) return;
    const int64_t U = uoff[e - s];
    if (U > ucap) {
        if (x == s) atomicOr(reinterpret_cast<unsigned long long *>(ctr + PC_OVF), (unsigned long long)OVF_UNITS);
        return;
    }
    if (x == s) {
        ufar[U] = 0;
        unear[U] = 0;
    }
    int64_t a = uoff[x - s], b = uoff[x - s + 1];
    for (int64_t u = a; u < b; u++) {
        unode[u] = (int32_t)x;
        uchunk[u] = (int32_t)(u - a);
    }
}

__device__ __forceinline__ bool mac_far_v(const float4 A, float Ra, const float4 B, float Rb, float theta2) {
    const float ex = __fadd_rn(__fsub_rn(A.x, B.x), __fsub_rn(A.y, B.y));
    const float ey = __fadd_rn(__fsub_rn(A.z, B.z), __fsub_rn(A.w, B.w));
    const float d2 = __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey));
    const float s = __fadd_rn(Ra, Rb);
    return __fmul_rn(d2, theta2) > __fmul_rn(s, s);
}

// pass 0: per-unit counts (ufar, unear), and each candidate's decisions in dec (one word
// per lane and unit: byte k holds candidate k * 32 + lane's far mask in the low nibble and
// its near mask in the high one, one bit per child slot); pass 1: the children written at
// the running totals plus the per-unit offsets, from dec without testing again.  A
// grid-stride loop over the level's units, one warp per unit; each lane loads its
// MAC_ROUNDS candidates, then their children, then tests them, so that the gathers of a
// unit are in flight together.
constexpr int MAC_ROUNDS = MAC_CHUNK / 32;
__global__ void __launch_bounds__(128) k_mac(const int64_t *Uptr, int pass, const int32_t *unode,
                                             const int32_t *uchunk, const int32_t *parent, const int4 *child,
                                             const float4 *hl, const float *R32, float theta2,
                                             const int64_t *near_start, const int32_t *near_cnt,
                                             const int32_t *near_idx_in, int64_t *ufar, int64_t *unear,
                                             int32_t *far_idx, int32_t *near_idx, int64_t far_cap, int64_t near_cap,
                                             uint32_t *dec, int64_t *ctr) {
    const unsigned full = 0xffffffffu;
    if (ctr[PC_OVF]) return;
    const int64_t n_units = *Uptr;
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t far0 = pass ? ctr[PC_FAR] : 0, near0 = pass ? ctr[PC_NEAR] : 0;
    for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n_units; u += nwarps) {
        const int32_t x = unode[u];
        const int32_t P = parent[x];
        // x is its parent's only child: against the only child of a near entry of P the
        // pair holds the parents' bodies and stays near without a test
        const bool only_child = child[P].y < 0;
        const int64_t qa = near_start[P] + (int64_t)uchunk[u] * MAC_CHUNK;
        const int qn = (int)min((int64_t)MAC_CHUNK, near_start[P] + (int64_t)near_cnt[P] - qa);
        int64_t fb = 0, nb = 0;
        if (pass) {
            // this unit's whole range must fit; otherwise flag and write nothing
            fb = far0 + ufar[u];
            nb = near0 + unear[u];
            const int64_t fe = far0 + ufar[u + 1], ne = near0 + unear[u + 1];
            const unsigned long long bad = (fe > far_cap ? OVF_FAR : 0) | (ne > near_cap ? OVF_NEAR : 0);
            if (bad) {
                if (lane == 0) atomicOr(reinterpret_cast<unsigned long long *>(ctr + PC_OVF), bad);
                continue;
            }
        }
        int32_t cand[MAC_ROUNDS];
#pragma unroll
        for (int k = 0; k < MAC_ROUNDS; k++) cand[k] = k * 32 + lane < qn ? near_idx_in[qa + k * 32 + lane] : -1;
        int4 c4[MAC_ROUNDS];
#pragma unroll
        for (int k = 0; k < MAC_ROUNDS; k++) c4[k] = cand[k] >= 0 ? child[cand[k]] : make_int4(-1, -1, -1, -1);
        uint32_t d = 0;
        if (pass) {
            d = dec[u * 32 + lane];
        } else {
            const float4 A = hl[x];
            const float Ra = R32[x];
#pragma unroll
            for (int k = 0; k < MAC_ROUNDS; k++) {
                const int cc[4] = {c4[k].x, c4[k].y, c4[k].z, c4[k].w};
                const bool inherit = only_child && cc[1] < 0;
                unsigned fm = 0, nm = 0;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    if (cc[j] < 0) continue;
                    if (!inherit && mac_far_v(A, Ra, hl[cc[j]], R32[cc[j]], theta2)) fm |= 1u << j;
                    else nm |= 1u << j;
                }
                d |= (fm | (nm << 4)) << (8 * k);
            }
            dec[u * 32 + lane] = d;
            const int nf = __reduce_add_sync(full, __popc(d & 0x0f0f0f0fu));
            const int nn = __reduce_add_sync(full, __popc(d & 0xf0f0f0f0u));
            if (lane == 0) {
                ufar[u] = nf;
                unear[u] = nn;
            }
            continue;
        }
        int64_t nf = 0, nn = 0;
#pragma unroll
        for (int k = 0; k < MAC_ROUNDS; k++) {
            const unsigned fm = (d >> (8 * k)) & 15u, nm = (d >> (8 * k + 4)) & 15u;
            const int myf = __popc(fm), myn = __popc(nm);
            int pf = myf, pn = myn;  // inclusive warp scans
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int tf = __shfl_up_sync(full, pf, o), tn = __shfl_up_sync(full, pn, o);
                if (lane >= o) {
                    pf += tf;
                    pn += tn;
                }
            }
            const int cc[4] = {c4[k].x, c4[k].y, c4[k].z, c4[k].w};
            int64_t a = fb + nf + (pf - myf), b = nb + nn + (pn - myn);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if ((fm >> j) & 1u) far_idx[a++] = cc[j];
                if ((nm >> j) & 1u) near_idx[b++] = cc[j];
            }
            nf += __shfl_sync(full, pf, 31);
            nn += __shfl_sync(full, pn, 31);
        }
    }
}

// Leaves below single-child chain levels 1 .. L: by the only-child rule every level
// under L keeps all of its parent's near entries (each mapped to its only child) and has
// no far entries, so a leaf's near list is its level-L ancestor's (node x + up) shifted
// down by up.  The level-L lists are the last block written, [NEAR - NEAR_LAST, NEAR);
// the leaf lists are that block copied after it, entry for entry (a flat copy: a warp per
// leaf left the ~6000-entry list of the widest halo leaf to one warp's dependent rounds),
// then each leaf takes its ancestor's offset within the block.
__global__ void k_chain_copy(int64_t up, int32_t *near_idx, int64_t near_cap, int64_t *ctr) {
    if (ctr[PC_OVF]) return;
    const int64_t n = ctr[PC_NEAR_LAST], dst = ctr[PC_NEAR], src = dst - n;
    if (dst + n > near_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            atomicOr(reinterpret_cast<unsigned long long *>(ctr + PC_OVF), (unsigned long long)OVF_NEAR);
        return;
    }
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        near_idx[dst + i] = (int32_t)(near_idx[src + i] - up);
}

__global__ void k_chain_leaf_offsets(int64_t nl, int64_t up, int64_t near_cap, int64_t *nstart, int32_t *ncnt,
                                     const int64_t *ctr) {
    const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nl) return;
    const int64_t n = ctr[PC_NEAR_LAST], dst = ctr[PC_NEAR];
    if (ctr[PC_OVF] || dst + n > near_cap) return;
    nstart[x] = dst + (nstart[x + up] - (dst - n));
    ncnt[x] = ncnt[x + up];
}

// The chain shortcut needs node x + l nl (levels 1 .. L) to have the single child
// x + (l - 1) nl, as Tree::build numbers them; a tree given from the host that does not
// flags OVF_CHAIN and is planned without the shortcut.
__global__ void k_chain_check(int64_t nl, int L, const int4 *child, int64_t *ctr) {
    int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nl) return;
    for (int l = 1; l <= L; l++) {
        const int4 c = child[x + l * nl];
        if (c.x != x + (l - 1) * nl || c.y >= 0) {
            atomicOr(reinterpret_cast<unsigned long long *>(ctr + PC_OVF), (unsigned long long)OVF_CHAIN);
            return;
        }
    }
}

__global__ void k_chain_leaf_close(int64_t *ctr) {
    if (ctr[PC_OVF]) return;
    ctr[PC_NEAR] += ctr[PC_NEAR_LAST];  // the leaf lists are as long as level L's
}

// The top levels of the tree (at most PLAN_SMALL nodes each, down to the first larger
// level) in one block: per level, each thread counts the far and near entries of its
// nodes, a block scan places them, and a second pass writes them in the same order as
// the multi-block pass (parent's near entry, child slot), with block barriers between
// the steps instead of a dozen launches per level.
constexpr int PLAN_SMALL = 256;
constexpr int PLAN_SMALL_THREADS = 1024;
struct PlanLevels {
    int64_t start[66];  // level_start of levels lo .. hi + 1 (relative index lv - lo)
    int lo, hi;
};

__device__ int plan_block_scan(int v, int *warp_tot, int *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
        int s = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
        int si = s;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= o) si += t;
        }
        if (lane < (int)(blockDim.x >> 5)) warp_tot[lane] = si - s;
        if (lane == 31) *total = si;
    }
    __syncthreads();
    int r = warp_tot[w] + inc - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(PLAN_SMALL_THREADS) k_mac_small_levels(
    PlanLevels L, const int32_t *__restrict__ parent, const int4 *__restrict__ child, const float4 *__restrict__ hl,
    const float *__restrict__ R32, float theta2, int64_t *fstart, int32_t *fcnt, int64_t *nstart, int32_t *ncnt,
    int32_t *far_idx, int32_t *near_idx, int64_t far_cap, int64_t near_cap, int64_t *ctr) {
    constexpr int PER = (PLAN_SMALL + PLAN_SMALL_THREADS - 1) / PLAN_SMALL_THREADS;
    constexpr int NW = PLAN_SMALL_THREADS / 32;
    const unsigned full = 0xffffffffu;
    __shared__ int cnt_f[PLAN_SMALL], cnt_n[PLAN_SMALL];
    __shared__ int warp_tot[32], tot_f, tot_n;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    // one warp walks node x's candidates 32 entries at a time (as k_mac does); pass 0
    // counts, pass 1 writes from (fb, nb) in list order
    auto walk = [&](int64_t x, int pass, int64_t fb, int64_t nb, int &nf_out, int &nn_out) {
        const int32_t P = parent[x];
        const bool only_child = child[P].y < 0;
        const int64_t qa = nstart[P], qe = qa + ncnt[P];
        const float4 A = hl[x];
        const float Ra = R32[x];
        int nf = 0, nn = 0;
        for (int64_t qb = qa; qb < qe; qb += 32 * MAC_ROUNDS) {
            int32_t cand[MAC_ROUNDS];
#pragma unroll
            for (int k = 0; k < MAC_ROUNDS; k++) cand[k] = qb + k * 32 + lane < qe ? near_idx[qb + k * 32 + lane] : -1;
            int4 c4[MAC_ROUNDS];
#pragma unroll
            for (int k = 0; k < MAC_ROUNDS; k++) c4[k] = cand[k] >= 0 ? child[cand[k]] : make_int4(-1, -1, -1, -1);
#pragma unroll
            for (int k = 0; k < MAC_ROUNDS; k++) {
                const int cc[4] = {c4[k].x, c4[k].y, c4[k].z, c4[k].w};
                const bool inherit = only_child && cc[1] < 0;
                unsigned fm = 0, nm = 0;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    if (cc[j] < 0) continue;
                    if (!inherit && mac_far_v(A, Ra, hl[cc[j]], R32[cc[j]], theta2)) fm |= 1u << j;
                    else nm |= 1u << j;
                }
                const int myf = __popc(fm), myn = __popc(nm);
                int pf = myf, pn = myn;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int tf = __shfl_up_sync(full, pf, o), tn = __shfl_up_sync(full, pn, o);
                    if (lane >= o) {
                        pf += tf;
                        pn += tn;
                    }
                }
                if (pass) {
                    int64_t a = fb + nf + (pf - myf), b = nb + nn + (pn - myn);
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        if ((fm >> j) & 1u) far_idx[a++] = cc[j];
                        if ((nm >> j) & 1u) near_idx[b++] = cc[j];
                    }
                }
                nf += __shfl_sync(full, pf, 31);
                nn += __shfl_sync(full, pn, 31);
            }
        }
        nf_out = nf;
        nn_out = nn;
    };
    for (int lv = L.hi; lv >= L.lo; lv--) {
        if (ctr[PC_OVF]) return;  // uniform: written by thread 0 before a barrier
        const int64_t s = L.start[lv - L.lo], e = L.start[lv - L.lo + 1], c = e - s;
        for (int64_t i = w; i < c; i += NW) {
            int nf, nn;
            walk(s + i, 0, 0, 0, nf, nn);
            if (lane == 0) {
                cnt_f[i] = nf;
                cnt_n[i] = nn;
            }
        }
        __syncthreads();
        // exclusive offsets of the nodes' entries (PER nodes per thread)
        int lf = 0, ln = 0, vf[PER], vn[PER];
        for (int k = 0; k < PER; k++) {
            const int64_t i = (int64_t)t * PER + k;
            vf[k] = i < c ? cnt_f[i] : 0;
            vn[k] = i < c ? cnt_n[i] : 0;
            lf += vf[k];
            ln += vn[k];
        }
        int of = plan_block_scan(lf, warp_tot, &tot_f);
        int on = plan_block_scan(ln, warp_tot, &tot_n);
        for (int k = 0; k < PER; k++) {
            const int64_t i = (int64_t)t * PER + k;
            if (i < c) {
                cnt_f[i] = of;  // now the node's offset within the level
                cnt_n[i] = on;
            }
            of += vf[k];
            on += vn[k];
        }
        __syncthreads();
        const int64_t base_f = ctr[PC_FAR], base_n = ctr[PC_NEAR];
        if (base_f + tot_f > far_cap || base_n + tot_n > near_cap) {
            if (t == 0)
                atomicOr(reinterpret_cast<unsigned long long *>(ctr + PC_OVF),
                         (unsigned long long)((base_f + tot_f > far_cap ? OVF_FAR : 0) |
                                              (base_n + tot_n > near_cap ? OVF_NEAR : 0)));
            return;
        }
        for (int64_t i = w; i < c; i += NW) {
            const int64_t fb = base_f + cnt_f[i], nb = base_n + cnt_n[i];
            int nf, nn;
            walk(s + i, 1, fb, nb, nf, nn);
            if (lane == 0) {
                fstart[s + i] = fb;
                fcnt[s + i] = nf;
                nstart[s + i] = nb;
                ncnt[s + i] = nn;
            }
        }
        __syncthreads();
        if (t == 0) {
            ctr[PC_FAR] = base_f + tot_f;
            ctr[PC_NEAR] = base_n + tot_n;
            ctr[PC_NEAR_LAST] = tot_n;
        }
        __syncthreads();
    }
}

// per node of the level: start (running total + first unit's offset) and count
__global__ void k_mac_node_lists(int64_t s, int64_t e, const int64_t *uoff, const int64_t *ufo, const int64_t *uno,
                                 const int64_t *ctr, int64_t *fstart, int32_t *fcnt, int64_t *nstart, int32_t *ncnt) {
    if (ctr[PC_OVF]) return;
    int64_t x = s + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= e) return;
    int64_t a = uoff[x - s], b = uoff[x - s + 1];
    fstart[x] = ctr[PC_FAR] + ufo[a];
    nstart[x] = ctr[PC_NEAR] + uno[a];
    fcnt[x] = (int32_t)(ufo[b] - ufo[a]);
    ncnt[x] = (int32_t)(uno[b] - uno[a]);
}

// after a level: advance the running totals by the level's far / near counts
__global__ void k_mac_advance(const int64_t *Uptr, const int64_t *ufo, const int64_t *uno, int64_t *ctr) {
    if (ctr[PC_OVF]) return;
    const int64_t U = *Uptr;
    ctr[PC_FAR] += ufo[U];
    ctr[PC_NEAR] += uno[U];
    ctr[PC_NEAR_LAST] = uno[U];
}

// ---------------------------------------------------------------- balanced build
// neighbors_geometric (lib.rs:382-423) + the 2:1 test of build_constrained
// (lib.rs:558-579): per leaf, the split point it asks for, or -1.
struct LevelSet {
    Level lv[64];
    int n;
};

__device__ __forceinline__ bool cells_adjacent_dev(const double *cx, const double *cy, const double *hw, int64_t a,
                                                   int64_t b) {
    double ha = hw[a], hb = hw[b];
    double mx = (ha != ha) ? hb : ((hb != hb) ? ha : (hb > ha ? hb : ha));
    double mn = (ha != ha) ? hb : ((hb != hb) ? ha : (hb < ha ? hb : ha));
    double ratio = __ddiv_rn(mx, mn);
    if (ratio > 8.0) return false;
    double dx = fabs(__dsub_rn(cx[a], cx[b])), dy = fabs(__dsub_rn(cy[a], cy[b]));
    double lim = __dadd_rn(__dadd_rn(ha, hb), 1e-15);
    return dx <= lim && dy <= lim;
}

__global__ void k_balance_splits(LevelSet ls, int64_t nl, const double *cx, const double *cy, const double *hw,
                                 const int32_t *bs, const int32_t *be, int64_t *mid_out, unsigned *status) {
    int64_t lid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (lid >= nl) return;
    double c_x = cx[lid], c_y = cy[lid], h = hw[lid];
    double d = __dmul_rn(h, 2.0);
    double px[8] = {__dadd_rn(c_x, d), __dadd_rn(c_x, d), c_x, __dsub_rn(c_x, d),
                    __dsub_rn(c_x, d), __dsub_rn(c_x, d), c_x, __dadd_rn(c_x, d)};
    double py[8] = {c_y, __dadd_rn(c_y, d), __dadd_rn(c_y, d), __dadd_rn(c_y, d),
                    c_y, __dsub_rn(c_y, d), __dsub_rn(c_y, d), __dsub_rn(c_y, d)};
    int64_t mid = -1;
    for (int k = 0; k < 8; k++) {
        int64_t best = -1;
        double bd = 1.7976931348623157e308;
        double qa = fabs(px[k]) + fabs(py[k]);
        bool qf = isfinite(px[k]) && isfinite(py[k]);
        for (int L = 0; L < ls.n; L++) {
            const Level &lv = ls.lv[L];
            double mg = margin(lv, qa);
            bool ok = level_query(lv, cx, cy, hw, px[k] - mg, px[k] + mg, py[k] - mg, py[k] + mg, qf, [&](int64_t o) {
                if (o == lid) return;
                double dx = fabs(__dsub_rn(px[k], cx[o])), dy = fabs(__dsub_rn(py[k], cy[o]));
                double lim = __dadd_rn(hw[o], 1e-15);
                if (!(dx <= lim && dy <= lim)) return;
                if (!cells_adjacent_dev(cx, cy, hw, lid, o)) return;
                double ex = __dsub_rn(px[k], cx[o]), ey = __dsub_rn(py[k], cy[o]);
                double dist = __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey));
                if (dist < bd) {  // candidates arrive in ascending id: ties keep the lowest id
                    bd = dist;
                    best = o;
                }
            });
            if (!ok) atomicOr(status, GX_DEV_STACK_OVERFLOW);
        }
        if (best >= 0) {
            double nhw = hw[best];
            if (h > __dmul_rn(nhw, 2.1)) {
                int64_t s = bs[lid], e = be[lid];
                if (e - s > 2) mid = (s + e) / 2;
                break;
            }
        }
    }
    mid_out[lid] = mid;
}

__global__ void k_flag_u8(int64_t nn, const uint8_t *len, uint8_t *flag) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nn) flag[i] = len[i] > 0;
}

__global__ void k_flag_i32(int64_t nn, const int32_t *cnt, uint8_t *flag) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nn) flag[i] = cnt[i] > 0;
}

}  // namespace

// Builds a BVH over nodes [s, e) into `storage` (grown as needed).
static int build_level(gx_ctx *ctx, int64_t s, int64_t e, DevBuf &storage, size_t offset_bytes, Level &L,
                       size_t *used_bytes) {
    int64_t cnt = e - s;
    int64_t nb = (cnt + BVH_B - 1) / BVH_B;
    if (nb < 1) nb = 1;
    int64_t p2 = 1;
    while (p2 < nb) p2 *= 2;
    size_t need = sizeof(double4) * (size_t)(2 * p2) + 64;
    L.s = s; L.e = e; L.p2 = p2;
    L.box = reinterpret_cast<double4 *>(static_cast<char *>(storage.p) + offset_bytes);
    L.cbox = nullptr;
    L.cmh = nullptr;
    L.cmax = 0.0;
    *used_bytes = need;
    (void)need;
    // status buffer: bytes [8,12) non-finite count, [16,24) max |c|+|hw|
    unsigned *nf = reinterpret_cast<unsigned *>(static_cast<char *>(ctx->status.p) + 8);
    double *ma = reinterpret_cast<double *>(static_cast<char *>(ctx->status.p) + 16);
    GX_CUDA(ctx, cudaMemsetAsync(nf, 0, 16, ctx->stream));
    k_bvh_leaves<<<gx_blocks(p2, 128), 128, 0, ctx->stream>>>(s, cnt, p2, dptr<double>(ctx->cx), dptr<double>(ctx->cy),
                                                             dptr<double>(ctx->hw), L.box, nf, ma);
    ctx->launches++;
    for (int64_t lo = p2 / 2; lo >= 1; lo /= 2) {
        k_bvh_up<<<gx_blocks(lo, 128), 128, 0, ctx->stream>>>(lo, 2 * lo, L.box);
        ctx->launches++;
    }
    GX_CUDA(ctx, cudaGetLastError());
    struct { unsigned nf; unsigned pad; double ma; } h{};
    GX_CUDA(ctx, cudaMemcpyAsync(&h, nf, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    L.brute = h.nf > 0;
    L.maxabs = h.ma;
    return GX_OK;
}

static size_t bvh_bytes(int64_t cnt) {
    int64_t nb = (cnt + BVH_B - 1) / BVH_B;
    if (nb < 1) nb = 1;
    int64_t p2 = 1;
    while (p2 < nb) p2 *= 2;
    return sizeof(double4) * (size_t)(2 * p2) + 256;
}

static int check_status(gx_ctx *ctx) {
    unsigned st = 0;
    GX_CUDA(ctx, cudaMemcpyAsync(&st, dptr<unsigned>(ctx->status), sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (st & GX_DEV_STACK_OVERFLOW) return gx_fail(ctx, GX_ERR_STATE, "list builder: traversal stack overflow");
    return GX_OK;
}

// V-list and U-list in the reference layout.
int gx_lists_build_ref(gx_ctx *ctx) {
    int64_t nn = ctx->n_nodes;
    GX_TRY(gx_ensure(ctx, ctx->vdata, sizeof(uint32_t) * GX_LIST_CAP * (size_t)(nn > 0 ? nn : 1)));
    GX_TRY(gx_ensure(ctx, ctx->udata, sizeof(uint32_t) * GX_LIST_CAP * (size_t)(nn > 0 ? nn : 1)));
    GX_TRY(gx_ensure(ctx, ctx->vlen, (size_t)(nn > 0 ? nn : 1)));
    GX_TRY(gx_ensure(ctx, ctx->ulen, (size_t)(nn > 0 ? nn : 1)));
    GX_CUDA(ctx, cudaMemsetAsync(ctx->vdata.p, 0xFF, sizeof(uint32_t) * GX_LIST_CAP * (size_t)nn, ctx->stream));
    GX_CUDA(ctx, cudaMemsetAsync(ctx->udata.p, 0xFF, sizeof(uint32_t) * GX_LIST_CAP * (size_t)nn, ctx->stream));
    GX_CUDA(ctx, cudaMemsetAsync(ctx->vlen.p, 0, (size_t)nn, ctx->stream));
    GX_CUDA(ctx, cudaMemsetAsync(ctx->ulen.p, 0, (size_t)nn, ctx->stream));
    GX_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(unsigned), ctx->stream));
    if (nn == 0) return GX_OK;
    const double *cx = dptr<double>(ctx->cx), *cy = dptr<double>(ctx->cy), *hw = dptr<double>(ctx->hw);
    // V-list, level by level
    for (int lv = 0; lv + 1 < ctx->n_levels; lv++) {
        int64_t s0 = ctx->level_start[lv], e0 = ctx->level_start[lv + 1];
        int64_t s1 = ctx->level_start[lv + 1], e1 = ctx->level_start[lv + 2];
        int64_t np = e1 - s1;
        size_t bb = bvh_bytes(np);
        GX_TRY(gx_ensure(ctx, ctx->scratch_a, 2 * bb + bb / 4 + 256));
        Level L;
        size_t used = 0;
        GX_TRY(build_level(ctx, s1, e1, ctx->scratch_a, 0, L, &used));
        L.cbox = reinterpret_cast<double4 *>(static_cast<char *>(ctx->scratch_a.p) + bb);
        L.cmh = reinterpret_cast<double *>(static_cast<char *>(ctx->scratch_a.p) + 2 * bb);
        double *cmax = reinterpret_cast<double *>(static_cast<char *>(ctx->status.p) + 24);
        GX_CUDA(ctx, cudaMemsetAsync(cmax, 0, sizeof(double), ctx->stream));
        k_cenv_leaves<<<gx_blocks(L.p2, 128), 128, 0, ctx->stream>>>(s1, np, L.p2, dptr<int4>(ctx->child), cx, cy, hw,
                                                                     L.cbox, L.cmh, cmax);
        ctx->launches++;
        for (int64_t lo = L.p2 / 2; lo >= 1; lo /= 2) {
            k_cenv_up<<<gx_blocks(lo, 128), 128, 0, ctx->stream>>>(lo, 2 * lo, L.cbox, L.cmh);
            ctx->launches++;
        }
        GX_CUDA(ctx, cudaMemcpyAsync(&L.cmax, cmax, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        k_vlist_node<<<gx_blocks(e0 - s0, 64), 64, 0, ctx->stream>>>(s0, e0, L, dptr<int32_t>(ctx->parent),
                                                                    dptr<int4>(ctx->child), cx, cy, hw,
                                                                    dptr<uint32_t>(ctx->vdata), dptr<uint8_t>(ctx->vlen),
                                                                    dptr<unsigned>(ctx->status));
        ctx->launches++;
        GX_CUDA(ctx, cudaGetLastError());
    }
    // U-list over the leaves
    {
        int64_t nl = ctx->level_start[1];
        GX_TRY(gx_ensure(ctx, ctx->scratch_a, bvh_bytes(nl)));
        Level L;
        size_t used = 0;
        GX_TRY(build_level(ctx, 0, nl, ctx->scratch_a, 0, L, &used));
        k_ulist<<<gx_blocks(nl, 128), 128, 0, ctx->stream>>>(L, cx, cy, hw, dptr<uint32_t>(ctx->udata),
                                                            dptr<uint8_t>(ctx->ulen), dptr<unsigned>(ctx->status));
        ctx->launches++;
        GX_CUDA(ctx, cudaGetLastError());
    }
    ctx->ref_lists_valid = true;
    return check_status(ctx);
}

// REF plan: P2P gather lists and the derivative-set id of every V pair.
int gx_plan_ref(gx_ctx *ctx) {
    int64_t nn = ctx->n_nodes;
    ctx->plan_ref_valid = false;
    if (nn == 0) { ctx->plan_ref_valid = true; return GX_OK; }
    GX_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(unsigned), ctx->stream));
    // ---- P2P gather lists
    int64_t nl = ctx->level_start[1];
    {
        GX_TRY(gx_ensure(ctx, ctx->scratch_c, sizeof(int64_t) * (size_t)(nl + 1) * 2));
        int64_t *cnt = dptr<int64_t>(ctx->scratch_c), *eoff = cnt + (nl + 1);
        GX_CUDA(ctx, cudaMemsetAsync(cnt + nl, 0, sizeof(int64_t), ctx->stream));
        k_gather_count<<<gx_blocks(nl, 256), 256, 0, ctx->stream>>>(nl, dptr<uint32_t>(ctx->udata),
                                                                    dptr<uint8_t>(ctx->ulen), cnt);
        GX_TRY(gx_exclusive_scan_i64(ctx, cnt, eoff, nl + 1));
        int64_t nk = 0;
        GX_CUDA(ctx, cudaMemcpyAsync(&nk, eoff + nl, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        // keys and their sort buffers: scratch_a (keys, alt), scratch_b (values, alt)
        GX_TRY(gx_ensure(ctx, ctx->scratch_a, sizeof(uint64_t) * (size_t)(nk + 1) * 2));
        GX_TRY(gx_ensure(ctx, ctx->scratch_b, sizeof(uint32_t) * (size_t)(nk + 1) * 2));
        uint64_t *keys = dptr<uint64_t>(ctx->scratch_a), *keys_alt = keys + (nk + 1);
        uint32_t *vals = dptr<uint32_t>(ctx->scratch_b), *vals_alt = vals + (nk + 1);
        k_gather_emit<<<gx_blocks(nl, 256), 256, 0, ctx->stream>>>(nl, dptr<uint32_t>(ctx->udata),
                                                                   dptr<uint8_t>(ctx->ulen), eoff, keys);
        int top = 1;
        while (top < 63 && ((int64_t)1 << top) <= nl) top++;
        bool alt = false;
        GX_TRY(gx_radix_sort_u64(ctx, keys, vals, nk, 0, 32 + top, keys_alt, vals_alt, &alt));
        const uint64_t *sk = alt ? keys_alt : keys;
        // per receiver: key range, list length, offsets, fill
        GX_TRY(gx_ensure(ctx, ctx->scratch_d, sizeof(int64_t) * (size_t)(nl + 1) * 2));
        int64_t *kstart = dptr<int64_t>(ctx->scratch_d), *len = kstart + (nl + 1);
        GX_CUDA(ctx, cudaMemsetAsync(len + nl, 0, sizeof(int64_t), ctx->stream));
        k_gather_ranges<<<gx_blocks(nl, 256), 256, 0, ctx->stream>>>(nl, sk, nk, kstart, len);
        GX_TRY(gx_ensure(ctx, ctx->p2p_off, sizeof(int64_t) * (size_t)(nl + 1)));
        int64_t *off = dptr<int64_t>(ctx->p2p_off);
        GX_TRY(gx_exclusive_scan_i64(ctx, len, off, nl + 1));
        int64_t tot = 0;
        GX_CUDA(ctx, cudaMemcpyAsync(&tot, off + nl, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        GX_TRY(gx_ensure(ctx, ctx->p2p_idx, sizeof(int32_t) * (size_t)(tot + 1)));
        k_gather_fill<<<gx_blocks(nl, 256), 256, 0, ctx->stream>>>(nl, sk, kstart, off, dptr<int32_t>(ctx->p2p_idx));
        ctx->launches += 6;
        ctx->n_p2p_pairs = tot;
        GX_CUDA(ctx, cudaGetLastError());
    }

    // ---- REF derivative plan
    GX_TRY(gx_ensure(ctx, ctx->ref_voff, sizeof(int64_t) * (size_t)(nn + 1)));  // V pair offsets per node
    int64_t *voff = dptr<int64_t>(ctx->ref_voff);
    GX_TRY(gx_ensure(ctx, ctx->scratch_c, sizeof(int64_t) * (size_t)(nn + 1)));
    int64_t *len64 = dptr<int64_t>(ctx->scratch_c);
    GX_CUDA(ctx, cudaMemsetAsync(len64 + nn, 0, sizeof(int64_t), ctx->stream));
    k_u8_to_i64<<<gx_blocks(nn, 256), 256, 0, ctx->stream>>>(dptr<uint8_t>(ctx->vlen), len64, nn);
    GX_TRY(gx_exclusive_scan_i64(ctx, len64, voff, nn + 1));
    int64_t np = 0;
    GX_CUDA(ctx, cudaMemcpyAsync(&np, voff + nn, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->n_v_pairs = np;
    GX_TRY(gx_ensure(ctx, ctx->ref_did, sizeof(int32_t) * (size_t)(np + 1)));
    if (np > 0) {
        // scratch_a: klo, khi, k_alt (3 x u64); scratch_b: pidx, pidx_alt (2 x u32) + heads;
        // scratch_d: pdx, pdy
        GX_TRY(gx_ensure(ctx, ctx->scratch_a, sizeof(uint64_t) * (size_t)np * 4));
        GX_TRY(gx_ensure(ctx, ctx->scratch_b, sizeof(uint32_t) * (size_t)np * 2 + sizeof(int32_t) * (size_t)np * 2 + 64));
        GX_TRY(gx_ensure(ctx, ctx->scratch_d, sizeof(double) * (size_t)np * 2));
        uint64_t *klo = dptr<uint64_t>(ctx->scratch_a), *khi = klo + np, *ka = khi + np, *kb = ka + np;
        uint32_t *pidx = dptr<uint32_t>(ctx->scratch_b), *palt = pidx + np;
        int32_t *head = reinterpret_cast<int32_t *>(palt + np), *hex = head + np;
        double *pdx = dptr<double>(ctx->scratch_d), *pdy = pdx + np;
        k_ref_pair_keys<<<gx_blocks(nn * GX_LIST_CAP, 256), 256, 0, ctx->stream>>>(
            nn, dptr<uint32_t>(ctx->vdata), dptr<uint8_t>(ctx->vlen), voff, dptr<double>(ctx->comx),
            dptr<double>(ctx->comy), klo, khi, pidx, pdx, pdy);
        ctx->launches++;
        // stable sort by lo, then by hi -> order (hi, lo, pair index)
        GX_CUDA(ctx, cudaMemcpyAsync(ka, klo, sizeof(uint64_t) * np, cudaMemcpyDeviceToDevice, ctx->stream));
        bool alt = false;
        GX_TRY(gx_radix_sort_u64(ctx, ka, pidx, np, 0, 64, kb, palt, &alt));
        uint32_t *p1 = alt ? palt : pidx;
        uint32_t *p1o = alt ? pidx : palt;
        k_gather_u64<<<gx_blocks(np, 256), 256, 0, ctx->stream>>>(p1, khi, ka, np);
        GX_TRY(gx_radix_sort_u64(ctx, ka, p1, np, 0, 64, kb, p1o, &alt));
        uint64_t *hs = alt ? kb : ka;
        uint32_t *p2 = alt ? p1o : p1;
        uint64_t *ls = alt ? ka : kb;
        k_gather_u64<<<gx_blocks(np, 256), 256, 0, ctx->stream>>>(p2, klo, ls, np);
        k_run_heads<<<gx_blocks(np, 256), 256, 0, ctx->stream>>>(hs, ls, np, head);
        int32_t nk = 0;
        GX_TRY(gx_exclusive_scan_i32(ctx, head, hex, np, &nk));
        GX_TRY(gx_ensure(ctx, ctx->scratch_c, sizeof(int32_t) * (size_t)(nk + 1)));
        int32_t *first = dptr<int32_t>(ctx->scratch_c);
        k_run_assign<<<gx_blocks(np, 256), 256, 0, ctx->stream>>>(head, hex, p2, np, dptr<int32_t>(ctx->ref_did), first);
        ctx->launches += 4;
        // polynomial table (host, by the reference's recurrence) and the derivative sets
        std::vector<double> poly;
        GX_TRY(gx_poly_table_host(ctx->p, ctx->eps, poly));
        int S = 2 * ctx->p + 1;
        GX_TRY(gx_ensure(ctx, ctx->scratch_e, sizeof(double) * poly.size()));
        GX_CUDA(ctx, cudaMemcpyAsync(ctx->scratch_e.p, poly.data(), sizeof(double) * poly.size(), cudaMemcpyHostToDevice,
                                     ctx->stream));
        GX_TRY(gx_ensure(ctx, ctx->ref_G, sizeof(double) * (size_t)nk * S * S));
        k_ref_derivs<<<gx_blocks(nk, 64), 64, 0, ctx->stream>>>(nk, first, pdx, pdy, dptr<double>(ctx->scratch_e),
                                                               ctx->p, ctx->eps, dptr<double>(ctx->ref_G));
        ctx->launches++;
        GX_CUDA(ctx, cudaGetLastError());
        GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        ctx->n_ref_keys = nk;
    }
    GX_TRY(gx_ensure(ctx, ctx->has_far_ref, (size_t)nn));
    k_flag_u8<<<gx_blocks(nn, 256), 256, 0, ctx->stream>>>(nn, dptr<uint8_t>(ctx->vlen), dptr<uint8_t>(ctx->has_far_ref));
    ctx->launches++;
    GX_TRY(check_status(ctx));
    ctx->plan_ref_valid = true;
    ctx->plan_p = ctx->p;
    ctx->plan_eps = ctx->eps;
    return GX_OK;
}

// ACCURATE plan: node radii from the resident bodies, then near/far lists top-down.
int gx_plan_accurate(gx_ctx *ctx) {
    int64_t nn = ctx->n_nodes;
    ctx->plan_acc_valid = false;
    if (nn == 0) { ctx->plan_acc_valid = true; return GX_OK; }
    if (!ctx->have_bodies) return gx_fail(ctx, GX_ERR_STATE, "accurate plan needs resident bodies");
    GX_TRY(gx_ensure(ctx, ctx->radius, sizeof(double) * (size_t)nn));
    double *R = dptr<double>(ctx->radius);
    int64_t nl = ctx->level_start[1];
    // per-node start/count for far and near lists
    GX_TRY(gx_ensure(ctx, ctx->far_off, sizeof(int64_t) * (size_t)nn + sizeof(int32_t) * (size_t)nn + 64));
    GX_TRY(gx_ensure(ctx, ctx->near_off, sizeof(int64_t) * (size_t)nn + sizeof(int32_t) * (size_t)nn + 64));
    int64_t *fstart = dptr<int64_t>(ctx->far_off);
    int32_t *fcnt = reinterpret_cast<int32_t *>(fstart + nn);
    int64_t *nstart = dptr<int64_t>(ctx->near_off);
    int32_t *ncnt = reinterpret_cast<int32_t *>(nstart + nn);
    const int64_t root = nn - 1;
    // FP32 MAC operands: (hi, lo) COMs (built with the tree aux) and radii rounded once
    const float thf = (float)ctx->theta;
    const float theta2 = thf * thf;
    GX_TRY(gx_ensure(ctx, ctx->radius32, sizeof(float) * (size_t)nn));
    float *R32 = dptr<float>(ctx->radius32);
    const float4 *hl = dptr<float4>(ctx->comhl);
    int64_t cmax = 1;
    for (int lv = 0; lv < ctx->n_levels; lv++)
        cmax = std::max<int64_t>(cmax, ctx->level_start[lv + 1] - ctx->level_start[lv]);
    // levels 1 .. L of single-child chains over the leaves: a level with as many nodes as
    // the one below groups nothing (each node is the one child of the node above it)
    const int64_t nl0 = ctx->level_start[1];
    int L = 0;
    while (L + 1 < ctx->n_levels && ctx->level_start[L + 2] - ctx->level_start[L + 1] == nl0) L++;
    ctx->chain_levels = L >= 2 ? L : 0;
    int lv_low = ctx->chain_levels;  // the lowest level the loop below processes
    // node radii, FP64 and rounded once to FP32: per level, or with the chain levels walked
    // by one thread per leaf and the top levels in one block
    auto radii = [&](int chain) -> int {
        k_radius_leaves<<<gx_blocks(nl * 32, 256), 256, 0, ctx->stream>>>(
            nl, dptr<double>(ctx->x), dptr<double>(ctx->y), dptr<double>(ctx->comx), dptr<double>(ctx->comy),
            dptr<int32_t>(ctx->bs), dptr<int32_t>(ctx->be), R);
        ctx->launches++;
        int lv = 1;
        if (chain >= 2) {
            k_radius_chain<<<gx_blocks(nl, 256), 256, 0, ctx->stream>>>(nl, chain, dptr<double>(ctx->comx),
                                                                       dptr<double>(ctx->comy), R);
            ctx->launches++;
            lv = chain + 1;
        }
        int top = ctx->n_levels;  // levels top .. n_levels - 1 go to one block
        while (top - 1 >= lv && ctx->level_start[top] - ctx->level_start[top - 1] <= RADIUS_TOP && top - 1 > ctx->n_levels - 65)
            top--;
        for (; lv < top; lv++) {
            const int64_t s = ctx->level_start[lv], e = ctx->level_start[lv + 1];
            k_radius_parents<<<gx_blocks(e - s, 128), 128, 0, ctx->stream>>>(s, e, dptr<int4>(ctx->child),
                                                                            dptr<double>(ctx->comx),
                                                                            dptr<double>(ctx->comy), R);
            ctx->launches++;
        }
        if (top < ctx->n_levels) {
            RadiusLevels RL;
            RL.lo = top;
            RL.hi = ctx->n_levels - 1;
            for (int l = RL.lo; l <= RL.hi + 1; l++) RL.start[l - RL.lo] = ctx->level_start[l];
            k_radius_top<<<1, RADIUS_TOP_THREADS, 0, ctx->stream>>>(RL, dptr<int4>(ctx->child),
                                                                   dptr<double>(ctx->comx), dptr<double>(ctx->comy), R);
            ctx->launches++;
        }
        k_to_f32<<<gx_blocks(nn, 256), 256, 0, ctx->stream>>>(nn, R, R32);
        ctx->launches++;
        GX_CUDA(ctx, cudaGetLastError());
        return GX_OK;
    };
    GX_TRY(radii(lv_low));
    // capacities: unit arrays and the far / near index arrays, kept from the last plan
    if (ctx->mac_ucap < 1024) ctx->mac_ucap = std::max<int64_t>(1024, nn);
    int64_t far_cap = std::max<int64_t>({(int64_t)(ctx->far_idx.bytes / sizeof(int32_t)), int64_t(1) << 20, 64 * nn,
                                         ctx->hint_far + ctx->hint_far / 8});
    int64_t near_cap = std::max<int64_t>({(int64_t)(ctx->near_idx.bytes / sizeof(int32_t)), int64_t(1) << 20, 64 * nn,
                                          ctx->hint_near + ctx->hint_near / 8});
    GX_TRY(gx_ensure(ctx, ctx->plan_ctr, sizeof(int64_t) * PC_N));
    int64_t *ctr = dptr<int64_t>(ctx->plan_ctr);
    int64_t hc[PC_N] = {0, 0, 0, 0};
    const unsigned gmac = (unsigned)(ctx->sm_count > 0 ? ctx->sm_count * 16 : 2432);  // grid-stride k_mac
    for (int attempt = 0;; attempt++) {
        if (attempt == 8) return gx_fail(ctx, GX_ERR_CAP_EXCEEDED, "accurate plan: list storage keeps overflowing");
        const int64_t ucap = ctx->mac_ucap;
        GX_TRY(gx_ensure(ctx, ctx->far_idx, sizeof(int32_t) * (size_t)far_cap));
        GX_TRY(gx_ensure(ctx, ctx->near_idx, sizeof(int32_t) * (size_t)near_cap));
        GX_TRY(gx_ensure(ctx, ctx->scratch_a, sizeof(int64_t) * (size_t)(cmax + 1) * 2));
        GX_TRY(gx_ensure(ctx, ctx->scratch_b, sizeof(int32_t) * (size_t)(ucap + 1) * 2));
        GX_TRY(gx_ensure(ctx, ctx->scratch_e, sizeof(int64_t) * (size_t)(ucap + 1) * 4));
        GX_TRY(gx_ensure(ctx, ctx->scratch_d, sizeof(uint32_t) * 32 * (size_t)(ucap + 1)));
        uint32_t *dec = dptr<uint32_t>(ctx->scratch_d);
        int64_t *nch = dptr<int64_t>(ctx->scratch_a), *uoff = nch + (cmax + 1);
        int32_t *unode = dptr<int32_t>(ctx->scratch_b), *uchunk = unode + (ucap + 1);
        int64_t *ufar = dptr<int64_t>(ctx->scratch_e), *unear = ufar + (ucap + 1), *ufo = unear + (ucap + 1),
                *uno = ufo + (ucap + 1);
        GX_CUDA(ctx, cudaMemsetAsync(fcnt, 0, sizeof(int32_t) * (size_t)nn, ctx->stream));
        GX_CUDA(ctx, cudaMemsetAsync(ncnt, 0, sizeof(int32_t) * (size_t)nn, ctx->stream));
        // root: near itself (near list {root} at index 0)
        hc[PC_FAR] = 0;
        hc[PC_NEAR] = 1;
        hc[PC_NEAR_LAST] = 0;
        hc[PC_OVF] = 0;
        const int64_t zero = 0;
        const int32_t one = 1, root32 = (int32_t)root;
        GX_CUDA(ctx, cudaMemcpyAsync(ctr, hc, sizeof(hc), cudaMemcpyHostToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(nstart + root, &zero, sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(ncnt + root, &one, sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(dptr<int32_t>(ctx->near_idx), &root32, sizeof(int32_t), cudaMemcpyHostToDevice,
                                     ctx->stream));
        if (lv_low >= 2) {
            k_chain_check<<<gx_blocks(nl0, 256), 256, 0, ctx->stream>>>(nl0, lv_low, dptr<int4>(ctx->child), ctr);
            ctx->launches++;
        }
        // the top levels of at most PLAN_SMALL nodes in one block, then the rest
        int lv_big = ctx->n_levels - 2;
        while (lv_big >= lv_low && ctx->level_start[lv_big + 1] - ctx->level_start[lv_big] <= PLAN_SMALL) lv_big--;
        if (lv_big < ctx->n_levels - 2) {
            PlanLevels PL;
            PL.lo = lv_big + 1;
            PL.hi = ctx->n_levels - 2;
            if (PL.hi - PL.lo + 2 > 66) return gx_fail(ctx, GX_ERR_CAP_EXCEEDED, "accurate plan: too many levels");
            for (int lv = PL.lo; lv <= PL.hi + 1; lv++) PL.start[lv - PL.lo] = ctx->level_start[lv];
            k_mac_small_levels<<<1, PLAN_SMALL_THREADS, 0, ctx->stream>>>(
                PL, dptr<int32_t>(ctx->parent), dptr<int4>(ctx->child), hl, R32, theta2, fstart, fcnt, nstart, ncnt,
                dptr<int32_t>(ctx->far_idx), dptr<int32_t>(ctx->near_idx), far_cap, near_cap, ctr);
            ctx->launches++;
            GX_CUDA(ctx, cudaGetLastError());
        }
        for (int lv = lv_big; lv >= lv_low; lv--) {
            const int64_t s = ctx->level_start[lv], e = ctx->level_start[lv + 1], c = e - s;
            // units: chunks of each node's candidate list
            k_mac_nchunks<<<gx_blocks(c + 1, 256), 256, 0, ctx->stream>>>(s, e, dptr<int32_t>(ctx->parent), ncnt, nch,
                                                                         ctr);
            GX_TRY(gx_exclusive_scan_i64(ctx, nch, uoff, c + 1));
            const int64_t *Ud = uoff + c;  // the level's unit count, on the device
            k_mac_units<<<gx_blocks(c, 256), 256, 0, ctx->stream>>>(s, e, uoff, ucap, unode, uchunk, ufar, unear,
                                                                   ctr);
            k_mac<<<gmac, 128, 0, ctx->stream>>>(Ud, 0, unode, uchunk, dptr<int32_t>(ctx->parent),
                                                 dptr<int4>(ctx->child), hl, R32, theta2, nstart, ncnt,
                                                 dptr<int32_t>(ctx->near_idx), ufar, unear, nullptr, nullptr, far_cap,
                                                 near_cap, dec, ctr);
            // ufar, unear -> ufo, uno (arrays ucap + 1 apart) in one scan
            GX_TRY(gx_exclusive_scan_i64_devn_multi(ctx, ufar, ufo, 2, ucap + 1, Ud, 1, ucap + 1));
            k_mac<<<gmac, 128, 0, ctx->stream>>>(Ud, 1, unode, uchunk, dptr<int32_t>(ctx->parent),
                                                 dptr<int4>(ctx->child), hl, R32, theta2, nstart, ncnt,
                                                 dptr<int32_t>(ctx->near_idx), ufo, uno, dptr<int32_t>(ctx->far_idx),
                                                 dptr<int32_t>(ctx->near_idx), far_cap, near_cap, dec, ctr);
            k_mac_node_lists<<<gx_blocks(c, 256), 256, 0, ctx->stream>>>(s, e, uoff, ufo, uno, ctr, fstart, fcnt,
                                                                        nstart, ncnt);
            k_mac_advance<<<1, 1, 0, ctx->stream>>>(Ud, ufo, uno, ctr);
            ctx->launches += 6;
            GX_CUDA(ctx, cudaGetLastError());
        }
        if (lv_low >= 2) {
            const int64_t up = ctx->level_start[lv_low];
            const unsigned gcopy = (unsigned)(ctx->sm_count > 0 ? ctx->sm_count * 8 : 1216);
            k_chain_copy<<<gcopy, 256, 0, ctx->stream>>>(up, dptr<int32_t>(ctx->near_idx), near_cap, ctr);
            k_chain_leaf_offsets<<<gx_blocks(nl0, 256), 256, 0, ctx->stream>>>(nl0, up, near_cap, nstart, ncnt, ctr);
            k_chain_leaf_close<<<1, 1, 0, ctx->stream>>>(ctr);
            ctx->launches += 3;
            GX_CUDA(ctx, cudaGetLastError());
        }
        GX_CUDA(ctx, cudaMemcpyAsync(hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (!hc[PC_OVF]) break;
        if (hc[PC_OVF] & OVF_CHAIN) {  // no shortcut for this tree; its radii per level
            ctx->chain_levels = lv_low = 0;
            GX_TRY(radii(0));
        }
        if (hc[PC_OVF] & OVF_UNITS) ctx->mac_ucap *= 4;
        if (hc[PC_OVF] & OVF_FAR) far_cap *= 4;
        if (hc[PC_OVF] & OVF_NEAR) near_cap *= 4;
    }
    const int64_t far_tot = hc[PC_FAR];
    ctx->hint_far = far_tot;
    ctx->hint_near = hc[PC_NEAR];
    ctx->n_near_pairs = ctx->n_levels > 1 ? hc[PC_NEAR_LAST] : 1;  // a one-leaf tree: the root near itself
    ctx->n_far_pairs = far_tot;
    GX_TRY(gx_ensure(ctx, ctx->has_far_acc, (size_t)nn));
    k_flag_i32<<<gx_blocks(nn, 256), 256, 0, ctx->stream>>>(nn, fcnt, dptr<uint8_t>(ctx->has_far_acc));
    ctx->launches++;
    GX_CUDA(ctx, cudaGetLastError());
    ctx->plan_acc_valid = true;
    ctx->plan_p = ctx->p;
    ctx->plan_eps = ctx->eps;
    ctx->plan_theta = ctx->theta;
    return GX_OK;
}

namespace {
// Near-list split.  A near pair (a <- s), s != a, is M2P when every target body sees the
// source leaf from at least d - R_a with (d - R_a) theta_w > R_s, else P2L when every
// source body lies at least d - R_s from com_a with (d - R_s) theta_w > R_a, else P2P; the
// leaf itself is P2P.  Tested in FP32 on the MAC's operands with separately rounded
// operations (the oracle's gxo_near_split makes the same decisions):
// d2 tw^2 > (R_s + tw R_a)^2, then d2 tw^2 > (R_a + tw R_s)^2.
__device__ __forceinline__ int near_kind(const float4 A, float Ra, const float4 B, float Rs, float tw, float tw2) {
    const float ex = __fadd_rn(__fsub_rn(A.x, B.x), __fsub_rn(A.y, B.y));
    const float ey = __fadd_rn(__fsub_rn(A.z, B.z), __fsub_rn(A.w, B.w));
    const float lhs = __fmul_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)), tw2);
    const float sm = __fadd_rn(Rs, __fmul_rn(tw, Ra));
    if (lhs > __fmul_rn(sm, sm)) return 1;
    const float sl = __fadd_rn(Ra, __fmul_rn(tw, Rs));
    return lhs > __fmul_rn(sl, sl) ? 2 : 0;
}

// Each leaf's list is cut into units of NS_CHUNK entries (unit = (leaf, chunk j, length)),
// one warp per unit, so that the widest halo leaves (lists of every leaf of the tree at
// 1M Plummer) spread over many warps like the short ones.  k_ns_kinds tags each entry
// with its kind (copied to scratch at the same offset, kind in bits 30-31) and counts the
// unit's kinds; k_ns_write sums the counts of the leaf's earlier units and of all of them
// and writes the unit's entries back, partitioned as [P2P | M2P | P2L] in list order.
constexpr int NS_CHUNK = 256;
constexpr int NS_ROUNDS = NS_CHUNK / 32;

__global__ void k_ns_nchunks(int64_t nl, const int32_t *ncnt, int64_t *nch) {
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a > nl) return;
    nch[a] = a == nl ? 0 : (ncnt[a] + NS_CHUNK - 1) / NS_CHUNK;
}

__global__ void k_ns_units(int64_t nl, const int32_t *ncnt, const int64_t *uoff, int4 *unit, int32_t *split_cnt) {
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nl) return;
    const int32_t c = ncnt[a];
    const int64_t u0 = uoff[a];
    for (int32_t j = 0; j * NS_CHUNK < c; j++) unit[u0 + j] = make_int4((int32_t)a, j, min(NS_CHUNK, c - j * NS_CHUNK), 0);
    if (c == 0) split_cnt[2 * a] = split_cnt[2 * a + 1] = 0;  // no unit writes them
}

__global__ void __launch_bounds__(128) k_ns_kinds(const int64_t *__restrict__ Ud, const int4 *__restrict__ unit,
                                                   const int64_t *__restrict__ nstart,
                                                   const int32_t *__restrict__ near_idx, int32_t *__restrict__ scratch,
                                                   const float4 *__restrict__ hl, const float *__restrict__ R32,
                                                   float tw, float tw2, int4 *__restrict__ ucnt) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t nu = *Ud, nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < nu; u += nwarps) {
        const int4 r = unit[u];
        const int32_t a = r.x;
        const int64_t s = nstart[a] + (int64_t)r.y * NS_CHUNK;
        int32_t v[NS_ROUNDS];
#pragma unroll
        for (int k = 0; k < NS_ROUNDS; k++) v[k] = k * 32 + lane < r.z ? near_idx[s + k * 32 + lane] : -1;
        const float4 A = hl[a];
        const float Ra = R32[a];
        int n1 = 0, n2 = 0;
#pragma unroll
        for (int k = 0; k < NS_ROUNDS; k++) {
            int kind = 0;
            if (v[k] >= 0) {
                if (v[k] != a) kind = near_kind(A, Ra, hl[v[k]], R32[v[k]], tw, tw2);
                scratch[s + k * 32 + lane] = v[k] | (kind << 30);  // node ids stay below 2^30 (checked by the host)
            }
            n1 += __popc(__ballot_sync(full, kind == 1));
            n2 += __popc(__ballot_sync(full, kind == 2));
        }
        if (lane == 0) ucnt[u] = make_int4(r.z - n1 - n2, n1, n2, 0);
    }
}

// tot[0..2] gets the three totals: per block, the leaf totals its warps met at chunk 0
__global__ void __launch_bounds__(128) k_ns_write(const int64_t *__restrict__ Ud, const int4 *__restrict__ unit,
                                                   const int64_t *__restrict__ uoff,
                                                   const int64_t *__restrict__ nstart,
                                                   const int32_t *__restrict__ scratch,
                                                   const int4 *__restrict__ ucnt, int32_t *__restrict__ near_idx,
                                                   int32_t *__restrict__ ncnt, int32_t *__restrict__ split_cnt,
                                                   unsigned long long *__restrict__ tot) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    __shared__ unsigned long long btot[3];
    if (threadIdx.x < 3) btot[threadIdx.x] = 0;
    __syncthreads();
    unsigned long long my[3] = {0, 0, 0};
    const int64_t nu = *Ud, nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < nu; u += nwarps) {
        const int4 r = unit[u];
        const int32_t a = r.x, j = r.y;
        const int64_t u0 = uoff[a], nua = uoff[a + 1] - u0;
        // counts of the leaf's units before this one (p) and of all of them (t)
        int p0 = 0, p1 = 0, p2 = 0, t0 = 0, t1 = 0, t2 = 0;
        for (int64_t i = lane; i < nua; i += 32) {
            const int4 c = ucnt[u0 + i];
            t0 += c.x;
            t1 += c.y;
            t2 += c.z;
            if (i < j) {
                p0 += c.x;
                p1 += c.y;
                p2 += c.z;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            p0 += __shfl_xor_sync(full, p0, o);
            p1 += __shfl_xor_sync(full, p1, o);
            p2 += __shfl_xor_sync(full, p2, o);
            t0 += __shfl_xor_sync(full, t0, o);
            t1 += __shfl_xor_sync(full, t1, o);
            t2 += __shfl_xor_sync(full, t2, o);
        }
        const int64_t s0 = nstart[a], s = s0 + (int64_t)j * NS_CHUNK;
        int o0 = p0, o1 = t0 + p1, o2 = t0 + t1 + p2;
#pragma unroll
        for (int k = 0; k < NS_ROUNDS; k++) {
            const bool ok = k * 32 + lane < r.z;
            const int32_t v = ok ? scratch[s + k * 32 + lane] : 0;
            const int kind = ok ? (v >> 30) & 3 : 3;
            const unsigned m0 = __ballot_sync(full, kind == 0), m1 = __ballot_sync(full, kind == 1),
                           m2 = __ballot_sync(full, kind == 2);
            if (ok) {
                const int pos = kind == 0 ? o0 + __popc(m0 & lt) : kind == 1 ? o1 + __popc(m1 & lt) : o2 + __popc(m2 & lt);
                near_idx[s0 + pos] = v & 0x3fffffff;
            }
            o0 += __popc(m0);
            o1 += __popc(m1);
            o2 += __popc(m2);
        }
        if (j == 0 && lane == 0) {
            ncnt[a] = t0;
            split_cnt[2 * a] = t1;
            split_cnt[2 * a + 1] = t2;
            my[0] += (unsigned long long)t0;
            my[1] += (unsigned long long)t1;
            my[2] += (unsigned long long)t2;
        }
    }
    if (lane == 0) {
        atomicAdd(&btot[0], my[0]);
        atomicAdd(&btot[1], my[1]);
        atomicAdd(&btot[2], my[2]);
    }
    __syncthreads();
    if (threadIdx.x < 3 && btot[threadIdx.x]) atomicAdd(tot + threadIdx.x, btot[threadIdx.x]);
}
}  // namespace

// The leaf-level split of the ACCURATE near lists (theta_w > 0; no counterpart in the
// reference, whose U-list pairs are all P2P, lib.rs:1395-1462): leaf pairs that fail the
// MAC but whose bodies are far on one side take the source leaf's multipole at each
// target body (M2P) or the source bodies into the target's local (P2L), both with
// truncation bounded by theta_w^(p+1) like the far pairs' by theta^(p+1).  Runs after
// gx_plan_accurate; the totals are read back by gx_plan_items.
int gx_plan_near_split(gx_ctx *ctx) {
    const int64_t nl = ctx->n_leaves, nn = ctx->n_nodes;
    if (nn >= ((int64_t)1 << 30)) return gx_fail(ctx, GX_ERR_CAP_EXCEEDED, "near-list split: 2^30 or more nodes");
    GX_TRY(gx_ensure(ctx, ctx->split_cnt, sizeof(int32_t) * 2 * (size_t)(nl > 0 ? nl : 1)));
    GX_TRY(gx_ensure(ctx, ctx->split_tot, sizeof(unsigned long long) * 4));
    GX_CUDA(ctx, cudaMemsetAsync(ctx->split_tot.p, 0, sizeof(unsigned long long) * 4, ctx->stream));
    if (nl > 0) {
        int64_t *nstart = dptr<int64_t>(ctx->near_off);
        int32_t *ncnt = reinterpret_cast<int32_t *>(nstart + nn);
        const float tw = (float)ctx->theta_w, tw2 = tw * tw;
        // units: at most one per leaf plus one per NS_CHUNK entries of the near-list storage
        const int64_t ncap = (int64_t)(ctx->near_idx.bytes / sizeof(int32_t));
        const int64_t ucap = nl + ncap / NS_CHUNK + 1;
        GX_TRY(gx_ensure(ctx, ctx->scratch_f, sizeof(int32_t) * (size_t)(ncap + 1)));
        GX_TRY(gx_ensure(ctx, ctx->scratch_a, sizeof(int64_t) * 2 * (size_t)(nl + 1)));
        GX_TRY(gx_ensure(ctx, ctx->scratch_b, sizeof(int4) * (size_t)ucap));
        GX_TRY(gx_ensure(ctx, ctx->scratch_d, sizeof(int4) * (size_t)ucap));
        int64_t *nch = dptr<int64_t>(ctx->scratch_a), *uoff = nch + (nl + 1);
        int4 *unit = dptr<int4>(ctx->scratch_b), *ucnt = dptr<int4>(ctx->scratch_d);
        k_ns_nchunks<<<gx_blocks(nl + 1, 256), 256, 0, ctx->stream>>>(nl, ncnt, nch);
        GX_TRY(gx_exclusive_scan_i64(ctx, nch, uoff, nl + 1));
        k_ns_units<<<gx_blocks(nl, 256), 256, 0, ctx->stream>>>(nl, ncnt, uoff, unit, dptr<int32_t>(ctx->split_cnt));
        const unsigned g = (unsigned)(ctx->sm_count > 0 ? ctx->sm_count * 16 : 2432);  // grid-stride, 4 warps a block
        k_ns_kinds<<<g, 128, 0, ctx->stream>>>(uoff + nl, unit, nstart, dptr<int32_t>(ctx->near_idx),
                                               dptr<int32_t>(ctx->scratch_f), dptr<float4>(ctx->comhl),
                                               dptr<float>(ctx->radius32), tw, tw2, ucnt);
        k_ns_write<<<g, 128, 0, ctx->stream>>>(uoff + nl, unit, uoff, nstart, dptr<int32_t>(ctx->scratch_f), ucnt,
                                               dptr<int32_t>(ctx->near_idx), ncnt, dptr<int32_t>(ctx->split_cnt),
                                               dptr<unsigned long long>(ctx->split_tot));
        ctx->launches += 4;
    }
    GX_CUDA(ctx, cudaGetLastError());
    return GX_OK;
}

namespace {
constexpr int P2P_K = 32;  // source leaves per P2P work item

// ancestor table: anc[level * nl + leaf] = the leaf's ancestor at that level
__global__ void k_ancestors(int64_t nl, int n_levels, const int32_t *parent, int32_t *anc) {
    int64_t leaf = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= nl) return;
    int32_t a = (int32_t)leaf;
    for (int j = 0; j < n_levels; j++) {
        anc[(int64_t)j * nl + leaf] = a;
        if (a >= 0) a = parent[a];
    }
}

// COM as FP32 (hi, lo): hi = fl(c), lo = fl(c - hi)
__global__ void k_comhl(int64_t nn, const double *comx, const double *comy, float4 *out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    float xh = (float)comx[i], yh = (float)comy[i];
    out[i] = make_float4(xh, (float)(comx[i] - (double)xh), yh, (float)(comy[i] - (double)yh));
}


// per leaf: number of items; start/count from either list layout.  With the near-list
// split (split != null) the leaf's P2P items are followed by its M2P items, whose
// source count is stored negated; split[2a] is the leaf's M2P count.
__global__ void k_items_count(int64_t nl, const int64_t *start, const int32_t *cnt, const int32_t *split,
                              int64_t *nitems) {
    int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a > nl) return;
    if (a == nl) { nitems[a] = 0; return; }
    int64_t c = cnt ? cnt[a] : start[a + 1] - start[a];
    int64_t cm = split ? split[2 * a] : 0;
    nitems[a] = (c + P2P_K - 1) / P2P_K + (cm + P2P_K - 1) / P2P_K;
}

// per leaf: number of M2P items (the compact list the M2P kernel runs over)
__global__ void k_m2p_items_count(int64_t nl, const int32_t *split, int64_t *n) {
    int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a > nl) return;
    n[a] = a == nl ? 0 : (split[2 * a] + P2P_K - 1) / P2P_K;
}

// one warp per leaf, lanes over its items: the widest halo leaves have ~1000 items
__global__ void k_items_fill(int64_t nl, const int64_t *start, const int32_t *cnt, const int32_t *split,
                             const int64_t *off, int32_t *leaf, int64_t *qb, int32_t *nq, const int64_t *m2p_off,
                             int32_t *m2p_list) {
    const int64_t a = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (a >= nl) return;
    const int64_t s0 = start[a];
    const int64_t c = cnt ? cnt[a] : start[a + 1] - start[a];
    const int64_t it0 = off[a], np = (c + P2P_K - 1) / P2P_K;
    for (int64_t k = lane; k < np; k += 32) {
        leaf[it0 + k] = (int32_t)a;
        qb[it0 + k] = s0 + k * P2P_K;
        nq[it0 + k] = (int32_t)min((int64_t)P2P_K, c - k * P2P_K);
    }
    const int64_t cm = split ? split[2 * a] : 0, nm = (cm + P2P_K - 1) / P2P_K;
    for (int64_t k = lane; k < nm; k += 32) {
        const int64_t it = it0 + np + k;
        leaf[it] = (int32_t)a;
        qb[it] = s0 + c + k * P2P_K;
        nq[it] = -(int32_t)min((int64_t)P2P_K, cm - k * P2P_K);
        m2p_list[m2p_off[a] + k] = (int32_t)it;
    }
}

// P2L units: per leaf the number of units of at most GX_P2L_UNIT source leaves (its P2L
// sources follow its P2P and M2P sources), and with the body-level P2L the number of
// units of at most GX_BODY_UNIT of its P2P rows (the masked bodies: length stored
// negated); then unit -> (leaf, first, length), every leaf-level unit (leaf by leaf)
// before every body-level one, so that each kernel's grid covers its own units only
__global__ void k_p2l_units_count(int64_t nl, const int32_t *split, int64_t *nunits) {
    int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a > nl) return;
    nunits[a] = a == nl ? 0 : (split[2 * a + 1] + GX_P2L_UNIT - 1) / GX_P2L_UNIT;
}

__global__ void k_body_units_count(int64_t nl, const int32_t *cnt, int64_t *nunits) {
    int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a > nl) return;
    nunits[a] = a == nl ? 0 : (cnt[a] + GX_BODY_UNIT - 1) / GX_BODY_UNIT;
}

__global__ void k_p2l_units_fill(int64_t nl, const int64_t *start, const int32_t *cnt, const int32_t *split, int body,
                                 const int64_t *leaf_u, const int64_t *body_u, int32_t *uleaf, int64_t *ustart,
                                 int32_t *ulen) {
    const int64_t a = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // a warp per leaf
    const int lane = threadIdx.x & 31;
    if (a >= nl) return;
    const int64_t s0 = start[a] + cnt[a] + split[2 * a];
    const int32_t c = split[2 * a + 1];
    const int64_t u0 = leaf_u[a];
    const int32_t nlu = (c + GX_P2L_UNIT - 1) / GX_P2L_UNIT;
    for (int32_t k = lane; k < nlu; k += 32) {
        uleaf[u0 + k] = (int32_t)a;
        ustart[u0 + k] = s0 + (int64_t)k * GX_P2L_UNIT;
        ulen[u0 + k] = min(GX_P2L_UNIT, c - k * GX_P2L_UNIT);
    }
    if (!body) return;
    const int32_t cp = cnt[a];
    const int64_t b0 = leaf_u[nl] + body_u[a];
    for (int32_t k = lane; k * GX_BODY_UNIT < cp; k += 32) {
        uleaf[b0 + k] = (int32_t)a;
        ustart[b0 + k] = start[a] + (int64_t)k * GX_BODY_UNIT;
        ulen[b0 + k] = -min(GX_BODY_UNIT, cp - k * GX_BODY_UNIT);
    }
}

// Body-level P2L masks.  Per body its FP32 offset from its leaf's COM (each axis the FP64
// difference rounded once), then per P2P row (a <- s), s != a, the bit set of s's bodies
// with |o_j + (com_s - com_a)|^2 theta_b^2 > R_a^2, in separately rounded FP32 operations
// (o_j and the leaf-pair shift each rounded once from FP64), so that the oracle decides
// every body alike.
__global__ void k_body_off32(int64_t nl, const double *x, const double *y, const double *comx, const double *comy,
                             const int32_t *bs, const int32_t *be, float2 *off) {
    const int64_t L = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (L >= nl) return;
    const double cx = comx[L], cy = comy[L];
    for (int32_t j = bs[L] + lane; j < be[L]; j += 32) {
        // the evaluation's sanitising (k_prepare, which runs after the plan: a position
        // beyond 1e100 or not finite counts as the origin), as the oracle applies it first
        double xj = x[j], yj = y[j];
        if (fabs(xj) > 1e100 || fabs(yj) > 1e100 || !isfinite(xj) || !isfinite(yj)) xj = yj = 0.0;
        off[j] = make_float2(__double2float_rn(__dsub_rn(xj, cx)), __double2float_rn(__dsub_rn(yj, cy)));
    }
}

__global__ void __launch_bounds__(128) k_body_masks(int64_t n_items, const int32_t *__restrict__ item_leaf,
                                                    const int64_t *__restrict__ item_qb,
                                                    const int32_t *__restrict__ item_nq,
                                                    const int32_t *__restrict__ near_idx,
                                                    const double *__restrict__ comx, const double *__restrict__ comy,
                                                    const int32_t *__restrict__ bs, const int32_t *__restrict__ be,
                                                    const float *__restrict__ R32, const float2 *__restrict__ off,
                                                    float tb2, uint32_t *__restrict__ mask) {
    // a warp per P2P item: lane k stages row k (first body, body count or 0 for the self
    // row, the FP32 shift) in shared memory, then the warp takes the rows eight at a time,
    // a lane per body, the eight rows' loads in flight together
    __shared__ __align__(16) int4 rmeta[4][32];
    const unsigned full = 0xffffffffu;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t it = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (it >= n_items) return;
    const int nq = item_nq[it];
    if (nq <= 0) return;  // an M2P item
    const int32_t a = item_leaf[it];
    const int64_t qb = item_qb[it];
    if (lane < nq) {
        const int32_t s = near_idx[qb + lane];
        const int32_t b0 = bs[s], ns = s == a ? 0 : be[s] - b0;
        const float hx = __double2float_rn(__dsub_rn(comx[s], comx[a]));
        const float hy = __double2float_rn(__dsub_rn(comy[s], comy[a]));
        rmeta[w][lane] = make_int4(b0, ns, __float_as_int(hx), __float_as_int(hy));
    }
    __syncwarp();
    const float ra = R32[a], ra2 = __fmul_rn(ra, ra);
    constexpr int G = 8;
    for (int k0 = 0; k0 < nq; k0 += G) {
        float2 o[G];
        bool live[G];
        float hx[G], hy[G];
#pragma unroll
        for (int g = 0; g < G; g++) {
            const int k = k0 + g;
            const int4 r = rmeta[w][k & 31];
            live[g] = k < nq && lane < r.y;
            hx[g] = __int_as_float(r.z);
            hy[g] = __int_as_float(r.w);
            o[g] = live[g] ? off[r.x + lane] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int g = 0; g < G; g++) {
            const float ex = __fadd_rn(o[g].x, hx[g]), ey = __fadd_rn(o[g].y, hy[g]);
            const float d2 = __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey));
            const unsigned m = __ballot_sync(full, live[g] && __fmul_rn(d2, tb2) > ra2);
            if (lane == 0 && k0 + g < nq) mask[qb + k0 + g] = m;
        }
    }
}

// M2L units: per node the number of units; then unit -> (node, first, length)
__global__ void k_m2l_units_count(int64_t nn, const int32_t *fcnt, int64_t *nunits) {
    int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a > nn) return;
    nunits[a] = a == nn ? 0 : (fcnt[a] + GX_M2L_UNIT - 1) / GX_M2L_UNIT;
}

__global__ void k_m2l_units_fill(int64_t nn, const int64_t *fstart, const int32_t *fcnt, const int64_t *node_u,
                                 int32_t *unode, int64_t *ustart, int32_t *ulen) {
    int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nn) return;
    int64_t u = node_u[a];
    for (int32_t k = 0; k < fcnt[a]; k += GX_M2L_UNIT, u++) {
        unode[u] = (int32_t)a;
        ustart[u] = fstart[a] + k;
        ulen[u] = min(GX_M2L_UNIT, fcnt[a] - k);
    }
}

__global__ void k_add_offsets(const int64_t *o, int64_t *dst, int64_t c, int64_t add) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < c) dst[i] = o[i] + add;
}
}  // namespace

int gx_add_offsets(gx_ctx *ctx, const int64_t *o, int64_t *dst, int64_t c, int64_t add) {
    k_add_offsets<<<gx_blocks(c, 256), 256, 0, ctx->stream>>>(o, dst, c, add);
    ctx->launches++;
    GX_CUDA(ctx, cudaGetLastError());
    return GX_OK;
}

// build_constrained (lib.rs:541-588) on the device: up to 10 rebuilds with split
// points; the per-leaf neighbour search runs on the GPU, the split-point set (a
// small sorted list) is kept on the host.
int gx_tree_balance(gx_ctx *ctx, int64_t n_max, const double bounds[4]) {
    std::vector<int64_t> splits;
    for (int iter = 0; iter < 10; iter++) {
        GX_TRY(gx_tree_rebuild_with_splits(ctx, n_max, bounds, splits));
        if (ctx->n_levels > 64) return gx_fail(ctx, GX_ERR_CAP_EXCEEDED, "balanced build: too many levels");
        LevelSet ls;
        ls.n = ctx->n_levels;
        size_t total = 0;
        for (int L = 0; L < ls.n; L++) total += bvh_bytes(ctx->level_start[L + 1] - ctx->level_start[L]);
        GX_TRY(gx_ensure(ctx, ctx->scratch_a, total));
        size_t off = 0;
        for (int L = 0; L < ls.n; L++) {
            size_t used = 0;
            GX_TRY(build_level(ctx, ctx->level_start[L], ctx->level_start[L + 1], ctx->scratch_a, off, ls.lv[L], &used));
            off += bvh_bytes(ctx->level_start[L + 1] - ctx->level_start[L]);
        }
        int64_t nl = ctx->n_leaves;
        GX_TRY(gx_ensure(ctx, ctx->scratch_b, sizeof(int64_t) * (size_t)nl));
        GX_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(unsigned), ctx->stream));
        k_balance_splits<<<gx_blocks(nl, 64), 64, 0, ctx->stream>>>(ls, nl, dptr<double>(ctx->cx), dptr<double>(ctx->cy),
                                                                   dptr<double>(ctx->hw), dptr<int32_t>(ctx->bs),
                                                                   dptr<int32_t>(ctx->be), dptr<int64_t>(ctx->scratch_b),
                                                                   dptr<unsigned>(ctx->status));
        ctx->launches++;
        GX_CUDA(ctx, cudaGetLastError());
        std::vector<int64_t> mids((size_t)nl);
        GX_CUDA(ctx, cudaMemcpyAsync(mids.data(), ctx->scratch_b.p, sizeof(int64_t) * (size_t)nl,
                                     cudaMemcpyDeviceToHost, ctx->stream));
        GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        GX_TRY(check_status(ctx));
        std::set<int64_t> have(splits.begin(), splits.end());
        bool added = false;
        for (int64_t m : mids) {
            if (m < 0 || have.count(m)) continue;
            have.insert(m);
            added = true;
        }
        if (!added) return GX_OK;
        splits.assign(have.begin(), have.end());
    }
    return gx_tree_rebuild_with_splits(ctx, n_max, bounds, splits);
}

// P2P work items of the current plan (REF gather lists or ACCURATE near lists).
int gx_plan_items(gx_ctx *ctx, bool accurate) {
    gx_ctx::Items &I = accurate ? ctx->items_acc : ctx->items_ref;
    I.valid = false;
    int64_t nl = ctx->n_leaves, nn = ctx->n_nodes;
    const int64_t *start;
    const int32_t *cnt;
    if (accurate) {
        start = dptr<int64_t>(ctx->near_off);
        cnt = reinterpret_cast<const int32_t *>(start + nn);
    } else {
        start = dptr<int64_t>(ctx->p2p_off);
        cnt = nullptr;
    }
    // the P2P items and (ACCURATE) the M2L units: counts and scans of both, one wait for
    // their two totals, then both fills
    const bool split = accurate && ctx->theta_w > 0.0;
    const bool body = split && nl > 0 && gx_body_split_on(ctx);  // body-level P2L units after the leaf-level ones
    if (accurate) ctx->plan_body_split = false;  // the masks follow these items (gx_plan_body_masks)
    const int32_t *scnt = split ? dptr<int32_t>(ctx->split_cnt) : nullptr;
    GX_TRY(gx_ensure(ctx, I.off, sizeof(int64_t) * (size_t)(nl + 1)));
    GX_TRY(gx_ensure(ctx, ctx->scratch_c, sizeof(int64_t) * (size_t)(nl + 1)));
    int64_t *nit = dptr<int64_t>(ctx->scratch_c);
    k_items_count<<<gx_blocks(nl + 1, 256), 256, 0, ctx->stream>>>(nl, start, cnt, scnt, nit);
    GX_TRY(gx_exclusive_scan_i64(ctx, nit, dptr<int64_t>(I.off), nl + 1));
    int64_t tot[5] = {0, 0, 0, 0, 0};
    unsigned long long stot[4] = {0, 0, 0, 0};
    gx_ctx::P2LUnits &PU = ctx->p2l_units;
    if (split) {
        GX_TRY(gx_ensure(ctx, ctx->m2p_off, sizeof(int64_t) * (size_t)(nl + 1)));
        GX_TRY(gx_ensure(ctx, ctx->scratch_e, sizeof(int64_t) * (size_t)(nl + 1)));  // free after the plan
        int64_t *nm = dptr<int64_t>(ctx->scratch_e);
        k_m2p_items_count<<<gx_blocks(nl + 1, 256), 256, 0, ctx->stream>>>(nl, scnt, nm);
        GX_TRY(gx_exclusive_scan_i64(ctx, nm, dptr<int64_t>(ctx->m2p_off), nl + 1));
        GX_CUDA(ctx, cudaMemcpyAsync(&tot[3], dptr<int64_t>(ctx->m2p_off) + nl, sizeof(int64_t),
                                     cudaMemcpyDeviceToHost, ctx->stream));
        ctx->launches++;
        GX_TRY(gx_ensure(ctx, PU.leaf_u, sizeof(int64_t) * (size_t)(nl + 1)));
        GX_TRY(gx_ensure(ctx, ctx->scratch_b, sizeof(int64_t) * (size_t)(nl + 1)));
        int64_t *npu = dptr<int64_t>(ctx->scratch_b);
        k_p2l_units_count<<<gx_blocks(nl + 1, 256), 256, 0, ctx->stream>>>(nl, scnt, npu);
        GX_TRY(gx_exclusive_scan_i64(ctx, npu, dptr<int64_t>(PU.leaf_u), nl + 1));
        GX_CUDA(ctx, cudaMemcpyAsync(&tot[2], dptr<int64_t>(PU.leaf_u) + nl, sizeof(int64_t), cudaMemcpyDeviceToHost,
                                     ctx->stream));
        GX_TRY(gx_ensure(ctx, PU.body_u, sizeof(int64_t) * (size_t)(nl + 1)));
        if (body) {
            k_body_units_count<<<gx_blocks(nl + 1, 256), 256, 0, ctx->stream>>>(nl, cnt, npu);
            GX_TRY(gx_exclusive_scan_i64(ctx, npu, dptr<int64_t>(PU.body_u), nl + 1));
            GX_CUDA(ctx, cudaMemcpyAsync(&tot[4], dptr<int64_t>(PU.body_u) + nl, sizeof(int64_t),
                                         cudaMemcpyDeviceToHost, ctx->stream));
            ctx->launches++;
        }
        GX_CUDA(ctx, cudaMemcpyAsync(stot, ctx->split_tot.p, sizeof(stot), cudaMemcpyDeviceToHost, ctx->stream));
        ctx->launches++;
    }
    GX_CUDA(ctx, cudaMemcpyAsync(&tot[0], dptr<int64_t>(I.off) + nl, sizeof(int64_t), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    gx_ctx::M2LUnits &U = ctx->m2l_units;
    const int64_t *fstart = accurate ? dptr<int64_t>(ctx->far_off) : nullptr;
    const int32_t *fcnt = accurate ? reinterpret_cast<const int32_t *>(fstart + nn) : nullptr;
    if (accurate) {
        GX_TRY(gx_ensure(ctx, U.node_u, sizeof(int64_t) * (size_t)(nn + 1)));
        GX_TRY(gx_ensure(ctx, ctx->m2l_cnt, sizeof(int64_t) * (size_t)(nn + 1)));
        int64_t *nu = dptr<int64_t>(ctx->m2l_cnt);
        k_m2l_units_count<<<gx_blocks(nn + 1, 256), 256, 0, ctx->stream>>>(nn, fcnt, nu);
        GX_TRY(gx_exclusive_scan_i64(ctx, nu, dptr<int64_t>(U.node_u), nn + 1));
        GX_CUDA(ctx, cudaMemcpyAsync(&tot[1], dptr<int64_t>(U.node_u) + nn, sizeof(int64_t), cudaMemcpyDeviceToHost,
                                     ctx->stream));
        ctx->launches++;
    }
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // the partial sums index items in 31 bits
    if (tot[0] >= ((int64_t)1 << 31)) return gx_fail(ctx, GX_ERR_CAP_EXCEEDED, "more than 2^31 P2P work items");
    GX_TRY(gx_ensure(ctx, I.leaf, sizeof(int32_t) * (size_t)(tot[0] + 1)));
    GX_TRY(gx_ensure(ctx, I.qb, sizeof(int64_t) * (size_t)(tot[0] + 1)));
    GX_TRY(gx_ensure(ctx, I.nq, sizeof(int32_t) * (size_t)(tot[0] + 1)));
    if (split) GX_TRY(gx_ensure(ctx, ctx->m2p_list, sizeof(int32_t) * (size_t)(tot[3] + 1)));
    k_items_fill<<<gx_blocks(nl * 32, 256), 256, 0, ctx->stream>>>(
        nl, start, cnt, scnt, dptr<int64_t>(I.off), dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb), dptr<int32_t>(I.nq),
        split ? dptr<int64_t>(ctx->m2p_off) : nullptr, split ? dptr<int32_t>(ctx->m2p_list) : nullptr);
    ctx->launches += 2;
    I.n = tot[0];
    if (accurate) {
        // the near-list split's state belongs to the ACCURATE plan: a REF plan made in
        // between (its own items) leaves it as it is
        ctx->n_m2p_items = split ? tot[3] : 0;
        PU.n = PU.n_leafu = PU.n_body = 0;
        ctx->n_m2p_pairs = ctx->n_p2l_pairs = 0;
    }
    if (split) {
        ctx->n_near_pairs = (int64_t)stot[0];
        ctx->n_m2p_pairs = (int64_t)stot[1];
        ctx->n_p2l_pairs = (int64_t)stot[2];
        const int64_t npu = tot[2] + (body ? tot[4] : 0);
        GX_TRY(gx_ensure(ctx, PU.leaf, sizeof(int32_t) * (size_t)(npu + 1)));
        GX_TRY(gx_ensure(ctx, PU.start, sizeof(int64_t) * (size_t)(npu + 1)));
        GX_TRY(gx_ensure(ctx, PU.len, sizeof(int32_t) * (size_t)(npu + 1)));
        k_p2l_units_fill<<<gx_blocks(nl * 32, 256), 256, 0, ctx->stream>>>(
            nl, start, cnt, scnt, body ? 1 : 0, dptr<int64_t>(PU.leaf_u), dptr<int64_t>(PU.body_u),
            dptr<int32_t>(PU.leaf), dptr<int64_t>(PU.start), dptr<int32_t>(PU.len));
        ctx->launches++;
        PU.n = npu;
        PU.n_leafu = tot[2];
        PU.n_body = body ? tot[4] : 0;
    }
    if (accurate) {
        const int64_t nun = tot[1];
        GX_TRY(gx_ensure(ctx, U.node, sizeof(int32_t) * (size_t)(nun + 1)));
        GX_TRY(gx_ensure(ctx, U.start, sizeof(int64_t) * (size_t)(nun + 1)));
        GX_TRY(gx_ensure(ctx, U.len, sizeof(int32_t) * (size_t)(nun + 1)));
        k_m2l_units_fill<<<gx_blocks(nn, 256), 256, 0, ctx->stream>>>(nn, fstart, fcnt, dptr<int64_t>(U.node_u),
                                                                      dptr<int32_t>(U.node), dptr<int64_t>(U.start),
                                                                      dptr<int32_t>(U.len));
        ctx->launches++;
        U.n = nun;
    }
    GX_CUDA(ctx, cudaGetLastError());
    I.valid = true;
    return GX_OK;
}

// The body-level P2L masks of the current ACCURATE plan (after gx_plan_items, whose P2L
// units include the body-level ones when gx_body_split_on).
int gx_plan_body_masks(gx_ctx *ctx) {
    ctx->plan_body_split = false;
    const int64_t nl = ctx->n_leaves, n = ctx->n_bodies;
    const gx_ctx::Items &I = ctx->items_acc;
    if (!gx_body_split_on(ctx) || nl == 0 || !I.valid) return GX_OK;
    const int64_t ncap = (int64_t)(ctx->near_idx.bytes / sizeof(int32_t));
    GX_TRY(gx_ensure(ctx, ctx->p2p_mask, sizeof(uint32_t) * (size_t)(ncap + 1)));
    GX_TRY(gx_ensure(ctx, ctx->body_off32, sizeof(float2) * (size_t)(n + 1)));
    k_body_off32<<<gx_blocks(nl * 32, 256), 256, 0, ctx->stream>>>(
        nl, dptr<double>(ctx->x), dptr<double>(ctx->y), dptr<double>(ctx->comx), dptr<double>(ctx->comy),
        dptr<int32_t>(ctx->bs), dptr<int32_t>(ctx->be), dptr<float2>(ctx->body_off32));
    const float tb = (float)ctx->theta_b, tb2 = tb * tb;
    if (I.n > 0)
        k_body_masks<<<gx_blocks(I.n * 32, 128), 128, 0, ctx->stream>>>(
            I.n, dptr<int32_t>(I.leaf), dptr<int64_t>(I.qb), dptr<int32_t>(I.nq), dptr<int32_t>(ctx->near_idx),
            dptr<double>(ctx->comx), dptr<double>(ctx->comy), dptr<int32_t>(ctx->bs), dptr<int32_t>(ctx->be),
            dptr<float>(ctx->radius32), dptr<float2>(ctx->body_off32), tb2, dptr<uint32_t>(ctx->p2p_mask));
    ctx->launches += 2;
    GX_CUDA(ctx, cudaGetLastError());
    ctx->plan_body_split = true;
    ctx->plan_theta_b = ctx->theta_b;
    return GX_OK;
}

// Per-tree auxiliary arrays: the leaves' ancestor table (direct L2L) and the FP32
// hi/lo node COMs (mixed-precision M2L offsets).
int gx_plan_tree_aux(gx_ctx *ctx) {
    int64_t nl = ctx->n_leaves, nn = ctx->n_nodes;
    int L = ctx->n_levels;
    GX_TRY(gx_ensure(ctx, ctx->anc, sizeof(int32_t) * (size_t)(nl > 0 ? nl : 1) * (size_t)(L > 0 ? L : 1)));
    GX_TRY(gx_ensure(ctx, ctx->comhl, sizeof(float4) * (size_t)(nn > 0 ? nn : 1)));
    if (nl > 0) {
        k_ancestors<<<gx_blocks(nl, 256), 256, 0, ctx->stream>>>(nl, L, dptr<int32_t>(ctx->parent), dptr<int32_t>(ctx->anc));
        k_comhl<<<gx_blocks(nn, 256), 256, 0, ctx->stream>>>(nn, dptr<double>(ctx->comx), dptr<double>(ctx->comy),
                                                             dptr<float4>(ctx->comhl));
        ctx->launches += 2;
        GX_CUDA(ctx, cudaGetLastError());
    }
    ctx->aux_valid = true;
    return GX_OK;
}
