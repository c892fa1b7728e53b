// gx_tree.cu -- device Tree::build (galax-core/src/lib.rs:163-361) and
// build_constrained (lib.rs:541-694).
//
// Bit-exactness rules: every value that decides topology or feeds a key is
// computed with separately rounded IEEE operations (__dmul_rn / __dadd_rn /
// __dsub_rn, which the compiler never contracts into FMA), in the reference's
// order: Morton normalisation, leaf mass and COM sums (body order), parent sums
// (child slot order), box centres and half-widths.
#include <algorithm>

#include "gx_internal.cuh"

namespace {

constexpr double kOneMinus = 1.0 - 1e-15;  // clamp bound of normalize (lib.rs:76)

// normalize (lib.rs:75-78): NaN clamps to NaN and casts to 0, like Rust `as u64`.
__device__ __forceinline__ uint64_t normalize_ref(double x, double lo, double hi) {
    double t = __ddiv_rn(__dsub_rn(x, lo), __dsub_rn(hi, lo));
    if (t < 0.0) t = 0.0;
    if (t > kOneMinus) t = kOneMinus;
    if (!(t > 0.0)) return 0ull;
    return __double2ull_rz(__dmul_rn(t, 2097152.0));
}

// The same cell index without the division.  The key uses t = RN(a / w), a = x - lo,
// w = hi - lo, only through floor(t * 2^21) clamped to [0, 2^21 - 1] (the clamp at
// 1 - 1e-15 and the clamp at 0 land in the end cells; NaN gives 0).  With
// iw = RN(1/w) (w > 0 finite, iw normal, formed once on the host) and |a/w| < 2,
// q = RN(a * iw) is within 1.5 * 2^-52 of a/w and RN(a/w) within 0.5 * 2^-52, so the two
// differ by at most 2^-51; times 2^21 (exact) that is 2^-30.  Hence when s = q * 2^21 lies
// farther than 2^-29 from an integer, floor(s) = floor(RN(a/w) * 2^21) exactly; values
// that near a cell boundary, and non-finite ones, take the correctly rounded division.
// One multiply instead of a correctly rounded FP64 division per coordinate.  iw21 =
// iw * 2^21 (exact), so s = RN(a * iw21) = RN(a * iw) * 2^21 wherever RN(a * iw) is
// normal; where it is not, s < 2^-29 and both take the division.  FP64 throughput on
// this part is a small fraction of FP32, so the tests on s (the window, the end cells,
// floor and the distance to the nearest integer) are integer operations on its bits,
// each equal to the FP64 comparison it replaces: for 1 <= s < 2^22 with exponent e the
// integer part is the significand shifted right by 52 - e and the fraction its low
// 52 - e bits, so "fraction in (2^-29, 1 - 2^-29)" is "low bits in (2^(23-e),
// 2^(52-e) - 2^(23-e))".
__device__ __forceinline__ uint64_t normalize_dev(double x, double lo, double hi, double iw21) {
    if (iw21 > 0.0) {
        const double s = __dmul_rn(__dsub_rn(x, lo), iw21);
        const int64_t b = __double_as_longlong(s);
        const uint64_t mag = (uint64_t)b & 0x7fffffffffffffffull;
        if (b <= 0) {                                            // s <= 0 (or a NaN with the sign bit)
            if (mag < 0x3ff0000000000000ull) return 0ull;        // -1 < s <= 0: the low cell
        } else if (b >= 0x413fffff80000000ll) {                  // s >= 2097151.5 (or +inf, NaN)
            if (b < 0x4150000000000000ll) return 2097151ull;     // s < 2^22: the top cell
        } else if (b < 0x3ff0000000000000ll) {                   // 0 < s < 1: cell 0 away from both ends
            if (b > 0x3e20000000000000ll && b < 0x3fefffffff000000ll) return 0ull;  // 2^-29 < s < 1 - 2^-29
        } else {                                                 // 1 <= s < 2097151.5
            const int sh = 52 - ((int)(b >> 52) - 1023);         // 32 .. 52
            const uint64_t sig = ((uint64_t)b & 0x000fffffffffffffull) | 0x0010000000000000ull;
            const uint64_t fr = sig & ((1ull << sh) - 1ull), eps = 1ull << (sh - 29);
            if (fr > eps && fr < (1ull << sh) - eps) return sig >> sh;
        }
    }
    return normalize_ref(x, lo, hi);
}

// spread_bits (lib.rs:85-93)
__device__ __forceinline__ uint64_t spread_dev(uint64_t v) {
    uint64_t x = v & ((1ull << 21) - 1);
    x = (x | (x << 16)) & 0x0000ffff0000ffffull;
    x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
    x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}

__global__ void k_morton(const double *__restrict__ x, const double *__restrict__ y, int64_t n, double x0, double x1,
                         double y0, double y1, double ixw21, double iyw21, uint64_t *__restrict__ keys,
                         uint32_t *__restrict__ idx) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    keys[i] = spread_dev(normalize_dev(x[i], x0, x1, ixw21)) | (spread_dev(normalize_dev(y[i], y0, y1, iyw21)) << 1);
    if (idx) idx[i] = (uint32_t)i;
}

}  // namespace

// RN(1 / (hi - lo)) * 2^21 for the division-free normalisation, or 0 (the division path)
// when the width is not a positive finite number whose reciprocal is a normal number with
// a finite 2^21 multiple
double gx_inv_width21(double lo, double hi) {
    const double w = hi - lo;
    if (!(w > 0.0) || !std::isfinite(w)) return 0.0;
    const double iw = 1.0 / w, iw21 = iw * 2097152.0;
    return (std::isfinite(iw21) && std::fpclassify(iw) == FP_NORMAL) ? iw21 : 0.0;
}

void gx_launch_morton(gx_ctx *ctx, const double *x, const double *y, int64_t n, const double bounds[4], uint64_t *keys,
                      uint32_t *idx) {
    k_morton<<<gx_blocks(n, 256), 256, 0, ctx->stream>>>(x, y, n, bounds[0], bounds[1], bounds[2], bounds[3],
                                                         gx_inv_width21(bounds[0], bounds[1]),
                                                         gx_inv_width21(bounds[2], bounds[3]), keys, idx);
    ctx->launches++;
}

namespace {

// gather of the seven body arrays (Tree::permute, lib.rs:146-161), na of them per
// launch: the index read once per body and a body's loads in flight together.  The
// launch's source arrays are meant to fit the L2 together (a gather from unsorted order
// touches them at random; from the previous step's order, almost in sequence).
struct Arrays7 {
    const double *in[7];
    double *out[7];
};
__global__ void k_permute7(const uint32_t *__restrict__ idx, int64_t n, int na, Arrays7 a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t j = idx[i];
    double v[7];
#pragma unroll
    for (int k = 0; k < 7; k++)
        if (k < na) v[k] = a.in[k][j];
#pragma unroll
    for (int k = 0; k < 7; k++)
        if (k < na) a.out[k][i] = v[k];
}

__device__ __forceinline__ double fmin_rs(double a, double b) { return (a != a) ? b : ((b != b) ? a : (b < a ? b : a)); }
__device__ __forceinline__ double fmax_rs(double a, double b) { return (a != a) ? b : ((b != b) ? a : (b > a ? b : a)); }

// leaf nodes (lib.rs:228-267); one thread per leaf, sums in body order.
__global__ void k_leaves(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ m,
                         const int32_t *__restrict__ rs, const int32_t *__restrict__ re, int64_t nl, double *cx,
                         double *cy, double *hw, double *mass, double *comx, double *comy, int32_t *bs, int32_t *be,
                         int4 *child, int32_t *parent, uint8_t *is_leaf) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= nl) return;
    int32_t s = rs[L], e = re[L];
    double ms = 0.0, sx = 0.0, sy = 0.0;
    double bx0 = 1.7976931348623157e308, bx1 = -1.7976931348623157e308;
    double by0 = 1.7976931348623157e308, by1 = -1.7976931348623157e308;
    for (int32_t i = s; i < e; i++) {
        double mm = m[i], xi = x[i], yi = y[i];
        ms = __dadd_rn(ms, mm);
        sx = __dadd_rn(sx, __dmul_rn(xi, mm));
        sy = __dadd_rn(sy, __dmul_rn(yi, mm));
        bx0 = fmin_rs(bx0, xi); bx1 = fmax_rs(bx1, xi);
        by0 = fmin_rs(by0, yi); by1 = fmax_rs(by1, yi);
    }
    double c_x = __dmul_rn(__dadd_rn(bx0, bx1), 0.5), c_y = __dmul_rn(__dadd_rn(by0, by1), 0.5);
    double h = __dadd_rn(__dmul_rn(fmax_rs(__dsub_rn(bx1, bx0), __dsub_rn(by1, by0)), 0.5), 1e-15);
    cx[L] = c_x; cy[L] = c_y; hw[L] = h; mass[L] = ms;
    comx[L] = ms > 0.0 ? __ddiv_rn(sx, ms) : c_x;
    comy[L] = ms > 0.0 ? __ddiv_rn(sy, ms) : c_y;
    bs[L] = s; be[L] = e;
    child[L] = make_int4(-1, -1, -1, -1);
    parent[L] = -1;
    is_leaf[L] = 1;
}

// leaf ranges of Tree::build: chunks of n_max
__global__ void k_chunk_ranges(int64_t n, int64_t n_max, int64_t nl, int32_t *rs, int32_t *re) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= nl) return;
    int64_t s = L * n_max, e = s + n_max < n ? s + n_max : n;
    rs[L] = (int32_t)s;
    re[L] = (int32_t)e;
}

// ---- parent rounds (lib.rs:269-354) ----
// The rounds run without host round trips: the level bounds, the shift and the round's
// segment and group counts live in a device state block, every kernel of a round reads
// them there, and the host only waits once per batch of rounds.  A round whose new
// level would not fit the node storage sets the overflow flag; the build is then redone
// with more storage.
enum {
    TS_S = 0, TS_E = 1, TS_C = 2, TS_SHIFT = 3, TS_NSEG = 4, TS_NG = 5, TS_FLAGS = 6, TS_ROUNDS = 7,
    TS_CHAIN_M = 8,  // min over adjacent leaves of the highest bit in which their first keys differ
    TS_CHAIN_L = 9,  // single-child rounds built by k_chain_rounds
    TS_N = 10
};
enum { TS_DONE = 1, TS_OVERFLOW = 2, TS_STUCK = 4 };
constexpr int TS_MAX_ROUNDS = 400;  // level starts kept: TS_MAX_ROUNDS + 2

constexpr int TS_SMALL = 2048;  // levels of at most this many nodes: k_rounds_small
// the multi-block round kernels do nothing once the build is over or the level is small
__device__ __forceinline__ bool round_off(const int64_t *st) { return st[TS_FLAGS] != 0 || st[TS_C] <= TS_SMALL; }

__global__ void k_round_heads(const int64_t *st, const uint64_t *__restrict__ keys, const int32_t *__restrict__ bs,
                              int64_t *head) {
    if (round_off(st)) return;
    const int64_t s = st[TS_S], c = st[TS_C];
    const unsigned sh = (unsigned)st[TS_SHIFT] & 63u;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c) return;
    uint64_t g = keys[bs[s + i]] >> sh;
    head[i] = (i == 0) ? 1 : (g != (keys[bs[s + i - 1]] >> sh));
}

__global__ void k_seg_start(const int64_t *st, const int64_t *head, const int64_t *segex, int64_t *segstart) {
    if (round_off(st)) return;
    const int64_t c = st[TS_C];
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c) return;
    if (head[i]) segstart[segex[i]] = i;
}

__global__ void k_seg_groups(const int64_t *st, const int64_t *segstart, int64_t *gcnt) {
    if (round_off(st)) return;
    const int64_t c = st[TS_C], nseg = st[TS_NSEG];
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nseg) return;
    int64_t len = ((k + 1 < nseg) ? segstart[k + 1] : c) - segstart[k];
    gcnt[k] = (len + 3) / 4;
}

// the new level must fit the node storage; its child slots start empty
__global__ void k_round_open(int64_t *st, int64_t cap_nodes, int4 *child) {
    if (round_off(st)) return;
    const int64_t e = st[TS_E], ng = st[TS_NG];
    if (e + ng > cap_nodes) {
        if (blockIdx.x == 0 && threadIdx.x == 0) st[TS_FLAGS] |= TS_OVERFLOW;
        return;
    }
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < ng) child[e + g] = make_int4(-1, -1, -1, -1);
}

__global__ void k_assign(const int64_t *st, const int64_t *head, const int64_t *segex, const int64_t *segstart,
                         const int64_t *goff, int32_t *parent, int32_t *child) {
    if (round_off(st)) return;
    const int64_t s = st[TS_S], e = st[TS_E], c = st[TS_C];
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c) return;
    int64_t seg = segex[i] + head[i] - 1;
    int64_t pos = i - segstart[seg];
    int64_t g = goff[seg] + pos / 4;
    parent[s + i] = (int32_t)(e + g);
    child[(e + g) * 4 + (pos & 3)] = (int32_t)(s + i);
}

// after a round: record the new level, move to it, and stop at a single node
__global__ void k_round_close(int64_t *st, int64_t *level_start) {
    if (round_off(st)) return;
    const int64_t e = st[TS_E], ng = st[TS_NG];
    if (st[TS_ROUNDS] >= TS_MAX_ROUNDS) {
        st[TS_FLAGS] |= TS_STUCK;
        return;
    }
    const int64_t r = ++st[TS_ROUNDS];
    level_start[r + 1] = e + ng;
    st[TS_S] = e;
    st[TS_E] = e + ng;
    st[TS_C] = ng;
    st[TS_SHIFT] += 2;
    if (ng <= 1) st[TS_FLAGS] |= TS_DONE;
}

// One parent of a round (lib.rs:298-335): mass, COM from the children's com x mass,
// centre of the union of the children's boxes, hw = 2 x the largest child hw, body range.
__device__ __forceinline__ void parent_fields_one(int64_t q, double *cx, double *cy, double *hw, double *mass,
                                                  double *comx, double *comy, int32_t *bs, int32_t *be,
                                                  const int4 *child, int32_t *parent, uint8_t *is_leaf) {
    int4 c4 = child[q];
    int cc[4] = {c4.x, c4.y, c4.z, c4.w};
    double ms = 0.0, sx = 0.0, sy = 0.0, mh = 0.0;
    double bx0 = 1.7976931348623157e308, bx1 = -1.7976931348623157e308;
    double by0 = 1.7976931348623157e308, by1 = -1.7976931348623157e308;
    int first = cc[0], last = cc[0];
    for (int k = 0; k < 4; k++) {
        int s = cc[k];
        if (s < 0) break;
        last = s;
        double cm = mass[s], h = hw[s], ccx = cx[s], ccy = cy[s];
        ms = __dadd_rn(ms, cm);
        sx = __dadd_rn(sx, __dmul_rn(comx[s], cm));
        sy = __dadd_rn(sy, __dmul_rn(comy[s], cm));
        if (h > mh) mh = h;
        double cl = __dsub_rn(ccx, h), cr = __dadd_rn(ccx, h);
        if (cl < bx0) bx0 = cl;
        if (cr > bx1) bx1 = cr;
        double cb = __dsub_rn(ccy, h), ct = __dadd_rn(ccy, h);
        if (cb < by0) by0 = cb;
        if (ct > by1) by1 = ct;
    }
    double c_x = __dmul_rn(__dadd_rn(bx0, bx1), 0.5), c_y = __dmul_rn(__dadd_rn(by0, by1), 0.5);
    cx[q] = c_x; cy[q] = c_y; hw[q] = __dmul_rn(mh, 2.0); mass[q] = ms;
    comx[q] = ms > 0.0 ? __ddiv_rn(sx, ms) : c_x;
    comy[q] = ms > 0.0 ? __ddiv_rn(sy, ms) : c_y;
    bs[q] = bs[first];
    be[q] = be[last];
    parent[q] = -1;
    is_leaf[q] = 0;
}

__global__ void k_parent_fields(const int64_t *st, double *cx, double *cy, double *hw, double *mass, double *comx,
                                double *comy, int32_t *bs, int32_t *be, const int4 *child, int32_t *parent,
                                uint8_t *is_leaf) {
    if (round_off(st)) return;
    const int64_t e = st[TS_E], ng = st[TS_NG];
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    parent_fields_one(e + g, cx, cy, hw, mass, comx, comy, bs, be, child, parent, is_leaf);
}

// Single-child rounds.  Round r groups consecutive nodes whose first bodies' keys agree
// after >> 2r; while every node of the level is its own group, the round makes one parent
// per node.  Starting from the leaves, that holds for rounds r = 1 .. m/2 exactly, m the
// smallest, over adjacent leaves, highest bit in which their first keys differ (below
// it the prefixes differ for every pair; at 2r > m one pair agrees).  k_chain_depth finds
// m; k_chain_rounds builds those rounds at once, a thread per leaf walking its chain
// (level l node x + l nl is the one parent of x + (l-1) nl, its fields by the same
// parent_fields_one as a round), and moves the round state past them, so the multi-block
// rounds start at the first round that groups.  At 1M Plummer that is the first eight
// rounds: 8 x 13 launches become 2.
__global__ void k_chain_depth(int64_t nl, const uint64_t *__restrict__ keys, const int32_t *__restrict__ bs,
                              int64_t *st) {
    __shared__ int wmin[8];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int m = 64;
    if (i >= 1 && i < nl) {
        const uint64_t d = keys[bs[i]] ^ keys[bs[i - 1]];
        m = d ? 63 - __clzll((long long)d) : -1;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        int b = wmin[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) b = min(b, wmin[w]);
        if (b < 64) atomicMin(reinterpret_cast<long long *>(st + TS_CHAIN_M), (long long)b);
    }
}

__global__ void k_chain_rounds(int64_t *st, int64_t *level_start, int64_t nl, int64_t cap_nodes, double *cx,
                               double *cy, double *hw, double *mass, double *comx, double *comy, int32_t *bs,
                               int32_t *be, int4 *child, int32_t *parent, uint8_t *is_leaf) {
    if (st[TS_FLAGS] != 0 || nl <= TS_SMALL) return;
    int64_t L = st[TS_CHAIN_M] >= 2 ? st[TS_CHAIN_M] / 2 : 0;
    L = min(L, cap_nodes / nl - 1);
    L = min(L, (int64_t)TS_MAX_ROUNDS - 2);
    if (L <= 0) return;
    const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x < nl) {
        for (int64_t l = 1; l <= L; l++) {
            const int64_t q = x + l * nl, c = x + (l - 1) * nl;
            child[q] = make_int4((int)c, -1, -1, -1);
            parent[c] = (int32_t)q;
            parent_fields_one(q, cx, cy, hw, mass, comx, comy, bs, be, child, parent, is_leaf);
        }
    }
    if (x == 0) {
        for (int64_t r = 1; r <= L; r++) level_start[r + 1] = (r + 1) * nl;
        st[TS_S] = L * nl;
        st[TS_E] = (L + 1) * nl;
        st[TS_C] = nl;
        st[TS_SHIFT] = 2 + 2 * L;
        st[TS_ROUNDS] = L;
        st[TS_CHAIN_L] = L;
    }
}

// The rounds of levels of at most TS_SMALL nodes, all in one block: each phase of a
// round is a loop over the level with a block barrier after it, so the tail of the
// tree (a dozen rounds at 1M) costs one launch instead of a dozen per round.
constexpr int RS_SMALL_THREADS = 1024;

__device__ int64_t block_excl_scan_small(int v, int *warp_tot, int *total) {
    // exclusive scan of one int per thread over RS_SMALL_THREADS threads
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
        int s = warp_tot[lane];
        int si = s;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= o) si += t;
        }
        warp_tot[lane] = si - s;
        if (lane == 31) *total = si;
    }
    __syncthreads();
    int r = warp_tot[w] + inc - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(RS_SMALL_THREADS) k_rounds_small(int64_t *st, int64_t *level_start, int64_t cap_nodes,
                                                                  const uint64_t *__restrict__ keys, double *cx,
                                                                  double *cy, double *hw, double *mass, double *comx,
                                                                  double *comy, int32_t *bs, int32_t *be, int32_t *child,
                                                                  int32_t *parent, uint8_t *is_leaf) {
    constexpr int PER = TS_SMALL / RS_SMALL_THREADS;  // items per thread
    __shared__ int head[TS_SMALL], segex[TS_SMALL], segstart[TS_SMALL], goff[TS_SMALL];
    __shared__ int warp_tot[32], tot;
    __shared__ int64_t sh_s, sh_e, sh_c, sh_flags, sh_rounds;
    __shared__ unsigned sh_shift;
    const int t = threadIdx.x;
    for (;;) {
        if (t == 0) {
            sh_s = st[TS_S];
            sh_e = st[TS_E];
            sh_c = st[TS_C];
            sh_flags = st[TS_FLAGS];
            sh_rounds = st[TS_ROUNDS];
            sh_shift = (unsigned)st[TS_SHIFT] & 63u;
        }
        __syncthreads();
        const int64_t s = sh_s, e = sh_e, c = sh_c;
        if (sh_flags != 0 || c > TS_SMALL) return;
        // heads and their exclusive scan (segment of each node)
        int loc[PER], lsum = 0;
        for (int k = 0; k < PER; k++) {
            const int i = t * PER + k;
            int h = 0;
            if (i < c) {
                const uint64_t g = keys[bs[s + i]] >> sh_shift;
                h = (i == 0) ? 1 : (g != (keys[bs[s + i - 1]] >> sh_shift));
                head[i] = h;
            }
            loc[k] = h;
            lsum += h;
        }
        int run = (int)block_excl_scan_small(lsum, warp_tot, &tot);
        const int nseg = tot;
        for (int k = 0; k < PER; k++) {
            const int i = t * PER + k;
            if (i < c) segex[i] = run;
            run += loc[k];
        }
        __syncthreads();
        for (int k = 0; k < PER; k++) {
            const int i = t * PER + k;
            if (i < c && head[i]) segstart[segex[i]] = i;
        }
        __syncthreads();
        // groups of at most 4 per segment and their exclusive scan
        lsum = 0;
        for (int k = 0; k < PER; k++) {
            const int j = t * PER + k;
            int g = 0;
            if (j < nseg) g = (int)((((j + 1 < nseg) ? segstart[j + 1] : (int)c) - segstart[j] + 3) / 4);
            loc[k] = g;
            lsum += g;
        }
        run = (int)block_excl_scan_small(lsum, warp_tot, &tot);
        const int ng = tot;
        for (int k = 0; k < PER; k++) {
            const int j = t * PER + k;
            if (j < nseg) goff[j] = run;
            run += loc[k];
        }
        if (e + ng > cap_nodes || sh_rounds >= TS_MAX_ROUNDS) {
            if (t == 0) st[TS_FLAGS] |= (e + ng > cap_nodes) ? TS_OVERFLOW : TS_STUCK;
            return;  // uniform: every thread saw the same counts
        }
        for (int g = t; g < ng; g += RS_SMALL_THREADS)
            reinterpret_cast<int4 *>(child)[e + g] = make_int4(-1, -1, -1, -1);
        __syncthreads();
        for (int k = 0; k < PER; k++) {
            const int i = t * PER + k;
            if (i >= c) continue;
            const int seg = segex[i] + head[i] - 1;
            const int pos = i - segstart[seg];
            const int64_t g = goff[seg] + pos / 4;
            parent[s + i] = (int32_t)(e + g);
            child[(e + g) * 4 + (pos & 3)] = (int32_t)(s + i);
        }
        __syncthreads();
        for (int g = t; g < ng; g += RS_SMALL_THREADS)
            parent_fields_one(e + g, cx, cy, hw, mass, comx, comy, bs, be, reinterpret_cast<const int4 *>(child),
                              parent, is_leaf);
        __syncthreads();
        if (t == 0) {
            const int64_t r = ++st[TS_ROUNDS];
            level_start[r + 1] = e + ng;
            st[TS_S] = e;
            st[TS_E] = e + ng;
            st[TS_C] = ng;
            st[TS_SHIFT] += 2;
            if (ng <= 1) st[TS_FLAGS] |= TS_DONE;
        }
        __syncthreads();
    }
}

// ---- build_constrained helpers (lib.rs:541-694) ----
// leaf ranges bounded by n_max and by the sorted split points (lib.rs:603-613):
// computed on the host from the split list, which is small.

}  // namespace

// Node storage with capacity growth (contents preserved).
static int ensure_nodes(gx_ctx *ctx, int64_t need) {
    struct F { DevBuf *b; size_t sz; };
    F f[] = {{&ctx->cx, 8}, {&ctx->cy, 8}, {&ctx->hw, 8}, {&ctx->mass, 8}, {&ctx->comx, 8}, {&ctx->comy, 8},
             {&ctx->bs, 4}, {&ctx->be, 4}, {&ctx->child, 16}, {&ctx->parent, 4}, {&ctx->is_leaf, 1}};
    for (auto &e : f) {
        size_t want = e.sz * (size_t)need;
        if (e.b->bytes >= want) continue;
        size_t nb = std::max(want, e.b->bytes * 2);
        void *p = nullptr;
        if (cudaMalloc(&p, nb) != cudaSuccess) return gx_fail(ctx, GX_ERR_ALLOC, "node storage allocation failed");
        if (e.b->p) {
            cudaMemcpyAsync(p, e.b->p, e.b->bytes, cudaMemcpyDeviceToDevice, ctx->stream);
            cudaStreamSynchronize(ctx->stream);
            cudaFree(e.b->p);
        }
        e.b->p = p;
        e.b->bytes = nb;
    }
    return GX_OK;
}

// Builds nodes from leaf ranges already in scratch (rs, re as int32), using ctx->keys
// (Morton keys of the tree-ordered bodies).
static int build_from_ranges(gx_ctx *ctx, const int32_t *rs, const int32_t *re, int64_t nl) {
    if (nl <= 0) return gx_fail(ctx, GX_ERR_STATE, "tree build: no leaves");
    // node storage: the last build's node count (a rebuild every step keeps it), else a
    // guess; a round that overflows it makes the build start again with more
    int64_t cap = std::max<int64_t>(nl * 4 + 64, ctx->hint_nodes + ctx->hint_nodes / 8 + 64);
    // per-round scratch: head, segex, segstart, gcnt, goff (int64, <= nl each)
    GX_TRY(gx_ensure(ctx, ctx->scratch_a, sizeof(int64_t) * (size_t)(nl + 1) * 5));
    GX_TRY(gx_ensure(ctx, ctx->tree_state, sizeof(int64_t) * (TS_N + TS_MAX_ROUNDS + 2)));
    int64_t *st = dptr<int64_t>(ctx->tree_state);
    int64_t *lstart = st + TS_N;  // level starts
    int64_t *head = dptr<int64_t>(ctx->scratch_a);
    int64_t *segex = head + (nl + 1), *segstart = segex + (nl + 1), *gcnt = segstart + (nl + 1),
            *goff = gcnt + (nl + 1);
    const unsigned gb = gx_blocks(nl, 256);
    int64_t hs[TS_N];
    for (int attempt = 0;; attempt++) {
        if (attempt == 8) return gx_fail(ctx, GX_ERR_ALLOC, "tree build: node storage keeps overflowing");
        GX_TRY(ensure_nodes(ctx, cap));
        k_leaves<<<gx_blocks(nl, 128), 128, 0, ctx->stream>>>(
            dptr<double>(ctx->x), dptr<double>(ctx->y), dptr<double>(ctx->m), rs, re, nl, dptr<double>(ctx->cx),
            dptr<double>(ctx->cy), dptr<double>(ctx->hw), dptr<double>(ctx->mass), dptr<double>(ctx->comx),
            dptr<double>(ctx->comy), dptr<int32_t>(ctx->bs), dptr<int32_t>(ctx->be), dptr<int4>(ctx->child),
            dptr<int32_t>(ctx->parent), dptr<uint8_t>(ctx->is_leaf));
        ctx->launches++;
        const int64_t init[TS_N] = {0, nl, nl, 2, 0, 0, nl > 1 ? 0 : TS_DONE, 0, 64, 0};
        const int64_t ls01[2] = {0, nl};
        GX_CUDA(ctx, cudaMemcpyAsync(st, init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
        GX_CUDA(ctx, cudaMemcpyAsync(lstart, ls01, sizeof(ls01), cudaMemcpyHostToDevice, ctx->stream));
        if (nl > TS_SMALL) {
            k_chain_depth<<<gx_blocks(nl, 256), 256, 0, ctx->stream>>>(nl, dptr<uint64_t>(ctx->keys),
                                                                      dptr<int32_t>(ctx->bs), st);
            k_chain_rounds<<<gx_blocks(nl, 128), 128, 0, ctx->stream>>>(
                st, lstart, nl, cap, dptr<double>(ctx->cx), dptr<double>(ctx->cy), dptr<double>(ctx->hw),
                dptr<double>(ctx->mass), dptr<double>(ctx->comx), dptr<double>(ctx->comy), dptr<int32_t>(ctx->bs),
                dptr<int32_t>(ctx->be), dptr<int4>(ctx->child), dptr<int32_t>(ctx->parent),
                dptr<uint8_t>(ctx->is_leaf));
            ctx->launches += 2;
        }
        // rounds in batches: the last build's round count first, then 8 at a time
        // multi-block rounds in batches (the last build's count first), each batch followed
        // by the single-block kernel for the small levels
        int batch = std::max(4, ctx->hint_big_rounds + 1);
        int issued = 0;
        for (;;) {
            for (int r = 0; r < batch; r++) {
                k_round_heads<<<gb, 256, 0, ctx->stream>>>(st, dptr<uint64_t>(ctx->keys), dptr<int32_t>(ctx->bs), head);
                GX_TRY(gx_exclusive_scan_i64_devn(ctx, head, segex, st + TS_C, 0, nl, st + TS_NSEG));
                k_seg_start<<<gb, 256, 0, ctx->stream>>>(st, head, segex, segstart);
                k_seg_groups<<<gb, 256, 0, ctx->stream>>>(st, segstart, gcnt);
                GX_TRY(gx_exclusive_scan_i64_devn(ctx, gcnt, goff, st + TS_NSEG, 0, nl, st + TS_NG));
                k_round_open<<<gb, 256, 0, ctx->stream>>>(st, cap, dptr<int4>(ctx->child));
                k_assign<<<gb, 256, 0, ctx->stream>>>(st, head, segex, segstart, goff, dptr<int32_t>(ctx->parent),
                                                      dptr<int32_t>(ctx->child));
                k_parent_fields<<<gx_blocks(nl, 128), 128, 0, ctx->stream>>>(
                    st, dptr<double>(ctx->cx), dptr<double>(ctx->cy), dptr<double>(ctx->hw), dptr<double>(ctx->mass),
                    dptr<double>(ctx->comx), dptr<double>(ctx->comy), dptr<int32_t>(ctx->bs), dptr<int32_t>(ctx->be),
                    dptr<int4>(ctx->child), dptr<int32_t>(ctx->parent), dptr<uint8_t>(ctx->is_leaf));
                k_round_close<<<1, 1, 0, ctx->stream>>>(st, lstart);
                ctx->launches += 7;
            }
            k_rounds_small<<<1, RS_SMALL_THREADS, 0, ctx->stream>>>(
                st, lstart, cap, dptr<uint64_t>(ctx->keys), dptr<double>(ctx->cx), dptr<double>(ctx->cy),
                dptr<double>(ctx->hw), dptr<double>(ctx->mass), dptr<double>(ctx->comx), dptr<double>(ctx->comy),
                dptr<int32_t>(ctx->bs), dptr<int32_t>(ctx->be), dptr<int32_t>(ctx->child), dptr<int32_t>(ctx->parent),
                dptr<uint8_t>(ctx->is_leaf));
            ctx->launches++;
            GX_CUDA(ctx, cudaGetLastError());
            issued += batch;
            GX_CUDA(ctx, cudaMemcpyAsync(hs, st, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream));
            GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            if (hs[TS_FLAGS] & TS_STUCK) return gx_fail(ctx, GX_ERR_STATE, "tree build did not converge");
            if (hs[TS_FLAGS] != 0) break;
            batch = 8;
        }
        if (!(hs[TS_FLAGS] & TS_OVERFLOW)) break;
        cap *= 2;
    }
    const int64_t rounds = hs[TS_ROUNDS];
    std::vector<int64_t> ls((size_t)rounds + 2);
    GX_CUDA(ctx, cudaMemcpyAsync(ls.data(), lstart, sizeof(int64_t) * ls.size(), cudaMemcpyDeviceToHost, ctx->stream));
    GX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->level_start.assign(ls.begin(), ls.end());
    ctx->hint_big_rounds = 0;  // multi-block rounds after the single-child ones
    for (size_t l = 0; l + 2 < ls.size(); l++)
        if (ls[l + 1] - ls[l] > TS_SMALL) ctx->hint_big_rounds++;
    ctx->hint_big_rounds = std::max<int64_t>(0, ctx->hint_big_rounds - hs[TS_CHAIN_L]);
    const int64_t nn = ls.back();
    ctx->n_nodes = nn;
    ctx->hint_nodes = nn;
    ctx->n_leaves = nl;
    ctx->n_levels = (int32_t)ctx->level_start.size() - 1;
    return GX_OK;
}

// Bodies must already be resident (ctx->x ... in input order).  Sorts them into
// Morton order on the device, then builds the node hierarchy.
int gx_tree_build_device(gx_ctx *ctx, int64_t n, int64_t n_max, const double bounds[4], int flags) {
    ctx->have_tree = false;
    ctx->plan_ref_valid = ctx->plan_acc_valid = ctx->ref_lists_valid = false;
    if (n <= 0) {
        ctx->n_nodes = ctx->n_leaves = 0;
        ctx->n_levels = 0;
        ctx->level_start.assign(1, 0);
        ctx->have_tree = true;
        return GX_OK;
    }
    if (n >= 0x7fffffffLL) return gx_fail(ctx, GX_ERR_CAP_EXCEEDED, "n must be < 2^31");
    // keys + permutation
    GX_TRY(gx_ensure(ctx, ctx->keys, sizeof(uint64_t) * n));
    GX_TRY(gx_ensure(ctx, ctx->scratch_b, sizeof(uint64_t) * n));               // keys alt
    GX_TRY(gx_ensure(ctx, ctx->scratch_c, sizeof(uint32_t) * n * 2));           // idx, idx alt
    uint64_t *keys = dptr<uint64_t>(ctx->keys), *keys_alt = dptr<uint64_t>(ctx->scratch_b);
    uint32_t *idx = dptr<uint32_t>(ctx->scratch_c), *idx_alt = idx + n;
    gx_launch_morton(ctx, dptr<double>(ctx->x), dptr<double>(ctx->y), n, bounds, keys, idx);
    GX_CUDA(ctx, cudaGetLastError());
    if (!(flags & GX_BUILD_BALANCED)) {
        bool alt = false;
        GX_TRY(gx_radix_sort_u64(ctx, keys, idx, n, 0, 42, keys_alt, idx_alt, &alt));
        if (alt) {
            GX_CUDA(ctx, cudaMemcpyAsync(keys, keys_alt, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, ctx->stream));
            idx = idx_alt;
        }
        // permute the seven arrays into their spare copies, then swap them in; as many
        // arrays per launch as fit in half of the 129 MB L2 together (all seven at 1M)
        DevBuf *arrs[7] = {&ctx->x, &ctx->y, &ctx->vx, &ctx->vy, &ctx->m, &ctx->ax, &ctx->ay};
        const int per = (int)std::max<int64_t>(1, std::min<int64_t>(7, ((int64_t)64 << 20) / (8 * n)));
        for (int k0 = 0; k0 < 7; k0 += per) {
            const int na = std::min(per, 7 - k0);
            Arrays7 a7{};
            for (int k = 0; k < na; k++) {
                GX_TRY(gx_ensure(ctx, ctx->body_alt[k0 + k], sizeof(double) * n));
                a7.in[k] = dptr<double>(*arrs[k0 + k]);
                a7.out[k] = dptr<double>(ctx->body_alt[k0 + k]);
            }
            k_permute7<<<gx_blocks(n, 256), 256, 0, ctx->stream>>>(idx, n, na, a7);
            ctx->launches++;
        }
        for (int k = 0; k < 7; k++) std::swap(*arrs[k], ctx->body_alt[k]);
        GX_TRY(gx_ensure(ctx, ctx->perm, sizeof(uint32_t) * n));
        GX_CUDA(ctx, cudaMemcpyAsync(ctx->perm.p, idx, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, ctx->stream));
        GX_CUDA(ctx, cudaGetLastError());
    }
    int64_t nl = (n + n_max - 1) / n_max;
    GX_TRY(gx_ensure(ctx, ctx->scratch_f, sizeof(int32_t) * (size_t)(2 * nl + 2) + 64));
    // scratch_f is also the radix-sort flag; the sort is finished at this point
    int32_t *rs = dptr<int32_t>(ctx->scratch_f), *re = rs + nl;
    k_chunk_ranges<<<gx_blocks(nl, 256), 256, 0, ctx->stream>>>(n, n_max, nl, rs, re);
    ctx->launches++;
    GX_CUDA(ctx, cudaGetLastError());
    ctx->n_bodies = n;
    GX_TRY(build_from_ranges(ctx, rs, re, nl));
    ctx->have_tree = true;
    return GX_OK;
}

// Rebuild with forced split points (build_with_constraints, lib.rs:592-694): no sort;
// keys from the resident bodies.  Exposed to the balanced builder in gx_lists.cu.
int gx_tree_rebuild_with_splits(gx_ctx *ctx, int64_t n_max, const double bounds[4], const std::vector<int64_t> &splits) {
    int64_t n = ctx->n_bodies;
    GX_TRY(gx_ensure(ctx, ctx->keys, sizeof(uint64_t) * n));
    GX_TRY(gx_ensure(ctx, ctx->scratch_c, sizeof(uint32_t) * n * 2));
    gx_launch_morton(ctx, dptr<double>(ctx->x), dptr<double>(ctx->y), n, bounds, dptr<uint64_t>(ctx->keys),
                     dptr<uint32_t>(ctx->scratch_c));
    std::vector<int32_t> hrs, hre;
    int64_t s = 0;
    size_t k = 0;
    while (s < n) {
        int64_t bound = std::min(s + n_max, n);
        while (k < splits.size() && splits[k] <= s) k++;
        int64_t e = (k < splits.size() && splits[k] < bound) ? splits[k] : bound;
        hrs.push_back((int32_t)s);
        hre.push_back((int32_t)e);
        s = e;
    }
    int64_t nl = (int64_t)hrs.size();
    GX_TRY(gx_ensure(ctx, ctx->scratch_f, sizeof(int32_t) * (size_t)(2 * nl + 2) + 64));
    int32_t *rs = dptr<int32_t>(ctx->scratch_f), *re = rs + nl;
    GX_CUDA(ctx, cudaMemcpyAsync(rs, hrs.data(), sizeof(int32_t) * nl, cudaMemcpyHostToDevice, ctx->stream));
    GX_CUDA(ctx, cudaMemcpyAsync(re, hre.data(), sizeof(int32_t) * nl, cudaMemcpyHostToDevice, ctx->stream));
    GX_TRY(build_from_ranges(ctx, rs, re, nl));
    ctx->have_tree = true;
    return GX_OK;
}
