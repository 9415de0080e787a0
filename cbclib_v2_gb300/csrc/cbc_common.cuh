/*
 * cbc_common.cuh — device code shared by the forward (cbc_draw_lines.cu) and the
 * adjoint (cbc_adjoint.cu): per-line records, the reference's walk in exact float
 * arithmetic, tile coverage, walk checkpoints and the span helpers.
 */
#ifndef CBC_COMMON_CUH
#define CBC_COMMON_CUH

#include <cuda_runtime.h>
#include <stdint.h>
#include <limits.h>
#include <atomic>
#include <string>
#include <type_traits>

#include "cbc_draw_lines.h"
#include "exact.cuh"

namespace cbc {

constexpr int kThreads = 256;
constexpr int kMaxChunk = 32;
constexpr int kDefaultTileW = 64;
constexpr int kDefaultTileH = 64;
constexpr int kDefaultChunk = 16;
constexpr int kFatal = (1 << CBC_ERR_INDEX) | (1 << CBC_ERR_CAPACITY) | (1 << CBC_ERR_RANGE) |
                       (1 << CBC_ERR_TERM);
constexpr int kInvalidEntry = INT_MIN;

/* ---- per-line walk record ------------------------------------------------------ */

enum : int { kAxisY = 1, kStepXNeg = 2, kStepYNeg = 4, kDrawable = 8, kFastDiv = 16 };

/* BresenhamPlotter state of one 2-D line (bresenham.hpp:243-263): the walk starts at
 * (x0, y0) = m_pt0 and ends when a coordinate reaches (x1, y1) = m_pt1 (step added). */
template <typename T>
struct alignas(16) LineRec {
    int32_t x0, y0, x1, y1;
    T t0, t1;        /* tangent pt1 - pt0; the normal is (t1, -t0)             */
    T len, len2;     /* amplitude(tangent), len * len                          */
    T w, ww;         /* width, width * width                                   */
    T te0, ne0;      /* tangent / normal errors at the walk start              */
    T px, py;        /* pt0, for the tile coverage only                        */
    T rlen, rww;     /* RN(1 / len), RN(1 / ww) for the division shortcut      */
    T ne_thr;        /* spans continue while |ne| < ne_thr (see span_threshold) */
    int32_t frame, flags;
    int32_t c0;      /* first in-frame long coordinate of the walk, in walk order  */
    int32_t ncols;   /* in-frame long coordinates of the walk                      */
    int32_t ck_base; /* index of the line's first walk checkpoint                  */
    int32_t pad;
};

/* the walk's exact iterator state at the first position whose walk index
 * (c - c0) * step_long reaches a multiple of kCkCols (cx = INT_MIN: the walk ends
 * first).  The lines render takes work items of kSeg columns, kCkCols / kSeg per
 * checkpoint: an item that starts past its checkpoint walks there first. */
constexpr int kCkCols = 16;
constexpr int kSeg = 8;
constexpr int kItemsPerCk = kCkCols / kSeg;
static_assert(kCkCols % kSeg == 0, "render items tile the checkpoint spacing");

template <typename T>
struct Checkpoint {
    int32_t cx, cy;
    T te, ne;
    int32_t line;   /* owning line                  */
    int32_t seg;    /* segment index within the line */
};

/* status block at the start of the workspace */
struct DevStatus {
    int flags;
    int strategy;                  /* CBC_STRATEGY_TILES / _LINES of the call */
    unsigned long long bad_line;
    long long idx_min;
    long long idx_max;
    unsigned long long pairs;      /* running pair cursor == pairs_needed */
    unsigned long long cks;        /* running checkpoint cursor            */
    unsigned long long work;       /* work-item counter of the lines render */
    unsigned long long nlong;      /* lines in the long-walk list of prep_kernel */
};

/* per line of the current render chunk */
template <typename T>
struct SlotParams {
    T ts, ns;           /* tangent / normal derivative along the short axis           */
    T len, len2, ww;
    T rlen, rww;
    T ne_thr;           /* span continuation threshold on |ne|                         */
    float rns;          /* ~1 / ns, for the span window estimate only                 */
    int ss;             /* step sign along the short axis (first span half)            */
    int axis;
    int fast;           /* len and ww in the range of the division shortcut            */
};

/* per line of the current render chunk: what the segment replays need */
template <typename T>
struct WalkSlot {
    T d0t, d1t, d0n, d1n;   /* step * tangent, step * normal per axis     */
    int sx, sy;
    int x1, y1;             /* walk end                                   */
    int c0, sa;             /* walk index = (c - c0) * sa                 */
    int k_lo, k_hi;         /* walk indices of the in-tile columns        */
    int ck_base;
    int ent_base;           /* entry pool index of walk index k_lo        */
    int seg_base;           /* first flattened segment item of this line  */
    int axis;
};

/* ---- arithmetic in the reference's rounding ----------------------------------- */

template <typename T> struct Ar;

template <> struct Ar<float> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt(float a) { return __fsqrt_rn(a); }
    static __device__ __forceinline__ float rcp(float a) { return __frcp_rn(a); }
    static __device__ __forceinline__ float from_int(int v) { return __int2float_rn(v); }
    static __device__ __forceinline__ float nterm(float ne, const SlotParams<float> &p) {
        return p.fast ? cbc_normal_term_r(ne, p.len, p.rlen) : cbc_normal_term(ne, p.len);
    }
    static __device__ __forceinline__ float error(float te, float nf, const SlotParams<float> &p) {
        return p.fast ? cbc_pixel_error_r(te, nf, p.len, p.len2, p.ww, p.rlen, p.rww)
                      : cbc_pixel_error(te, nf, p.len, p.len2, p.ww);
    }
    /* error() where 0 <= te <= len^2 (no tangent term): the correctly rounded nf / ww */
    static __device__ __forceinline__ float error_inside(float nf, const SlotParams<float> &p) {
        return p.fast ? cbc_div(nf, p.ww, p.rww) : cbc_div_ieee(nf, p.ww);
    }
    template <int K>
    static __device__ __forceinline__ float profile(float x) { return cbc_profile_f32(K, x); }
    /* the same, the gaussian reading its table from `tab` (null: the global table) */
    template <int K>
    static __device__ __forceinline__ float profile_tab(float x, const float *tab) {
        if (K == CBC_GAUSSIAN && tab) return cbc_gaussian_tab(x, tab);
        return cbc_profile_f32(K, x);
    }
    static __device__ __forceinline__ bool fast_range(float v) {
        return v >= CBC_DIV_LO && v <= CBC_DIV_HI;
    }
};

template <> struct Ar<double> {
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ double sqrt(double a) { return __dsqrt_rn(a); }
    static __device__ __forceinline__ double rcp(double a) { return __drcp_rn(a); }
    static __device__ __forceinline__ double from_int(int v) { return (double)v; }
    /* the quotients below: from the correctly rounded reciprocal (cbc_ddiv) when len
     * and ww lie in its range, otherwise the IEEE division; the same double either way */
    static __device__ __forceinline__ double qdiv(double a, double b, double rb, int fast) {
        return fast ? cbc_ddiv(a, b, rb) : __ddiv_rn(a, b);
    }
    /* normal_error: T accumulator fed with pow(b, 2) = fl(b * b) (bresenham.hpp:284-289) */
    static __device__ __forceinline__ double nterm(double ne, const SlotParams<double> &p) {
        double b = qdiv(ne, p.len, p.rlen, p.fast);
        return __dmul_rn(b, b);
    }
    /* error(): fl(fl(fl(a * a) + nf) / ww) (bresenham.hpp:291-296) */
    static __device__ __forceinline__ double error(double te, double nf,
                                                   const SlotParams<double> &p) {
        double m1 = -te, m2 = __dsub_rn(te, p.len2);
        double ta = (m1 < m2) ? m2 : m1;
        if (ta < 0.0) ta = 0.0;
        double a = qdiv(ta, p.len, p.rlen, p.fast);
        return qdiv(__dadd_rn(__dmul_rn(a, a), nf), p.ww, p.rww, p.fast);
    }
    static __device__ __forceinline__ double error_inside(double nf, const SlotParams<double> &p) {
        return qdiv(nf, p.ww, p.rww, p.fast);
    }
    template <int K>
    static __device__ __forceinline__ double profile(double x) { return cbc_profile_f64(K, x); }
    template <int K>
    static __device__ __forceinline__ double profile_tab(double x, const float *) {
        return cbc_profile_f64(K, x);
    }
    static __device__ __forceinline__ bool fast_range(double v) {
        return v >= CBC_DDIV_LO && v <= CBC_DDIV_HI;
    }
};

/* ---- line preparation ---------------------------------------------------------- */

template <typename T>
__device__ __forceinline__ bool finite_val(T v) { return isfinite(v); }

/* The span loops of draw_line_2d continue while normal_error < width^2, with
 * normal_error = fl(fl(ne / len)^2) (bresenham.hpp:369-380).  That is a monotone
 * function of |ne| (round-to-nearest is monotone and odd), so the test equals
 * |ne| < ne_thr for ne_thr = the least non-negative float with
 * fl(fl(ne_thr / len)^2) >= ww, found by bisection over the float bit patterns. */
template <typename T>
__device__ T span_threshold(T len, T ww);

template <>
__device__ inline float span_threshold<float>(float len, float ww)
{
    auto reaches = [&](unsigned u) {
        const float b = __fdiv_rn(__uint_as_float(u), len);
        return __fmul_rn(b, b) >= ww;
    };
    /* the answer lies within a few ulps of sqrt(ww) * len: search there first */
    const float g = __fmul_rn(__fsqrt_rn(ww), len);
    unsigned u = __float_as_uint(g);
    if (g > 0.0f && u < 0x7f000000u) {
        if (reaches(u)) {
            for (int i = 0; i < 16; i++, u--)
                if (u == 0u || !reaches(u - 1u)) return __uint_as_float(u);
        } else {
            for (int i = 0; i < 16; i++)
                if (reaches(++u)) return __uint_as_float(u);
        }
    }
    unsigned lo = 0u, hi = 0x7f800000u;              /* f(+inf) = inf >= ww */
    while (lo < hi) {
        unsigned mid = lo + ((hi - lo) >> 1);
        float b = __fdiv_rn(__uint_as_float(mid), len);
        if (__fmul_rn(b, b) >= ww) hi = mid; else lo = mid + 1;
    }
    return __uint_as_float(lo);
}

template <>
__device__ inline double span_threshold<double>(double len, double ww)
{
    unsigned long long lo = 0ull, hi = 0x7ff0000000000000ull;
    while (lo < hi) {
        unsigned long long mid = lo + ((hi - lo) >> 1);
        double b = __ddiv_rn(__longlong_as_double((long long)mid), len);
        if (__dmul_rn(b, b) >= ww) hi = mid; else lo = mid + 1;
    }
    return __longlong_as_double((long long)lo);
}

/* BresenhamPlotter(line, long(ceil(width) + 1)) (bresenham.hpp:243-253) plus begin()
 * (:255-263).  Returns false for lines that draw nothing in the reference (zero
 * length, non-positive width) or whose walk is not defined (non-finite values). */
template <typename T>
__device__ bool build_rec(const T *ln, LineRec<T> &r, bool &too_long)
{
    using A = Ar<T>;
    too_long = false;
    T p0x = ln[0], p0y = ln[1], p1x = ln[2], p1y = ln[3], w = ln[4];
    if (!(finite_val(p0x) && finite_val(p0y) && finite_val(p1x) && finite_val(p1y) &&
          finite_val(w)))
        return false;
    if (!(w > T(0))) return false;            /* error() is +inf for width <= 0 */
    T t0 = A::sub(p1x, p0x), t1 = A::sub(p1y, p0y);
    int axis = (fabs(t0) < fabs(t1)) ? 1 : 0; /* first max |tau| */
    T mag = A::add(A::mul(t0, t0), A::mul(t1, t1));
    T len = A::sqrt(mag);
    if (!(len > T(0))) return false;          /* error() is NaN everywhere */
    T ceilw = A::add(ceil(w), T(1));
    if (!(ceilw < T(1e9))) return false;
    T tn0 = A::div(t0, len), tn1 = A::div(t1, len);
    T scale = fabs(A::div(ceilw, axis ? tn1 : tn0));
    int sx = (p1x >= p0x) ? 1 : -1, sy = (p1y >= p0y) ? 1 : -1;
    T a0 = round(A::sub(p0x, A::mul(scale, tn0)));
    T a1 = round(A::sub(p0y, A::mul(scale, tn1)));
    T b0 = round(A::add(p1x, A::mul(scale, tn0)));
    T b1 = round(A::add(p1y, A::mul(scale, tn1)));
    const T lim = T(1 << 30);
    if (!(fabs(a0) < lim && fabs(a1) < lim && fabs(b0) < lim && fabs(b1) < lim)) {
        too_long = true;
        return false;
    }
    r.x0 = (int32_t)a0;
    r.y0 = (int32_t)a1;
    r.x1 = (int32_t)b0 + sx;
    r.y1 = (int32_t)b1 + sy;
    long long walk = axis ? (long long)r.y1 - r.y0 : (long long)r.x1 - r.x0;
    if (walk < 0) walk = -walk;
    /* spans reach width * len / |t_long| pixels off the line along the short axis */
    T span = A::div(A::mul(w, len), fabs(axis ? t1 : t0));
    if (walk > CBC_MAX_WALK || !(span < T(CBC_MAX_WALK))) {
        too_long = true;
        return false;
    }
    T d0 = A::sub(A::from_int(r.x0), p0x), d1 = A::sub(A::from_int(r.y0), p0y);
    r.t0 = t0;
    r.t1 = t1;
    r.len = len;
    r.len2 = A::mul(len, len);
    r.w = w;
    r.ww = A::mul(w, w);
    r.te0 = A::add(A::mul(t0, d0), A::mul(t1, d1));
    r.ne0 = A::add(A::mul(t1, d0), A::mul(-t0, d1));
    r.px = p0x;
    r.py = p0y;
    r.rlen = A::rcp(len);
    r.rww = A::rcp(r.ww);
    bool fast = A::fast_range(len) && A::fast_range(r.ww);
    r.ne_thr = span_threshold<T>(len, r.ww);
    r.flags = axis | (sx < 0 ? kStepXNeg : 0) | (sy < 0 ? kStepYNeg : 0) | kDrawable |
              (fast ? kFastDiv : 0);
    return true;
}

struct Geometry {
    int H, W;
    int tile_w, tile_h;
    int tiles_x, tiles_y;
};

/* Conservative tile coverage of the pixels the walk can draw.  The walk covers the
 * long-axis range [m_pt0, m_pt1) exactly; at long coordinate c its centre pixel lies
 * within 1 px of the line and its spans stop where |normal distance| >= width, i.e.
 * within width * len / |t_long| of the line along the short axis. */
template <typename T>
struct Coverage {
    int a, sa;          /* long axis, walk direction along it                          */
    int lmin, lmax;     /* long-axis range of the walk inside the frame                */
    int TA, TS;         /* tile extents along the long / short axis                    */
    int ext_s;
    float ps, pa, slope, hw;

    __device__ bool init(const LineRec<T> &r, const Geometry &g) {
        a = r.flags & kAxisY;
        const int sxs = (r.flags & kStepXNeg) ? -1 : 1, sys = (r.flags & kStepYNeg) ? -1 : 1;
        sa = a ? sys : sxs;
        int first = a ? r.y0 : r.x0;
        int last = (a ? r.y1 : r.x1) - sa;
        lmin = max(min(first, last), 0);
        const int ext_a = a ? g.H : g.W;
        ext_s = a ? g.W : g.H;
        lmax = min(max(first, last), ext_a - 1);
        TA = a ? g.tile_h : g.tile_w;
        TS = a ? g.tile_w : g.tile_h;
        const float ta = (float)(a ? r.t1 : r.t0), ts = (float)(a ? r.t0 : r.t1);
        pa = (float)(a ? r.py : r.px);
        ps = (float)(a ? r.px : r.py);
        slope = ts / ta;
        hw = (float)r.w * (float)r.len / fabsf(ta) + 2.0f;
        return lmin <= lmax;
    }
    /* tile rows (short-axis tile indices) [j0, j1] of tile column ti; false if none */
    __device__ bool rows(int ti, int &j0, int &j1) const {
        int ca = max(lmin, ti * TA), cb = min(lmax, ti * TA + TA - 1);
        float s0 = ps + ((float)ca - pa) * slope, s1 = ps + ((float)cb - pa) * slope;
        float smin = fminf(s0, s1) - hw, smax = fmaxf(s0, s1) + hw;
        if (!(smax >= 0.0f) || !(smin <= (float)(ext_s - 1))) return false;
        j0 = max(0, (int)floorf(fmaxf(smin, -1.0f))) / TS;
        j1 = min(ext_s - 1, (int)floorf(fminf(smax, (float)ext_s))) / TS;
        return j0 <= j1;
    }
    __device__ int bin(int ti, int tj, const Geometry &g) const {
        return a ? (ti * g.tiles_x + tj) : (tj * g.tiles_x + ti);
    }
};

/* the reference's outer-walk step (LineIterator::update + operator++, bresenham.hpp:
 * 205-220 and 98-111, for the single axis pair of 2-D) */
template <typename T>
struct Walker {
    int cx, cy;
    T te, ne;
    int sx, sy;
    T d0t, d1t, d0n, d1n;   /* step * tangent, step * normal per axis */

    __device__ void init(const LineRec<T> &r) {
        sx = (r.flags & kStepXNeg) ? -1 : 1;
        sy = (r.flags & kStepYNeg) ? -1 : 1;
        d0t = sx > 0 ? r.t0 : -r.t0;
        d1t = sy > 0 ? r.t1 : -r.t1;
        d0n = sx > 0 ? r.t1 : -r.t1;
        d1n = sy > 0 ? -r.t0 : r.t0;
    }
    /* the normal errors of the three candidate moves from the current position:
     * x only, y only, both (the last is exx + d1n, as the reference adds it) */
    struct Next {
        T exx, eyy, exy;
        bool nx, ny;
    };
    /* decisions at the current position: step x (nx) and / or y (ny) */
    __device__ __forceinline__ Next decide() const {
        using A = Ar<T>;
        Next n;
        n.exx = A::add(ne, d0n);
        n.eyy = A::add(ne, d1n);
        n.exy = A::add(n.exx, d1n);
        if constexpr (sizeof(T) == sizeof(double)) {
            /* |a| < |b| as the order of the sign-cleared bit patterns (integer pipe) */
            constexpr long long m = 0x7fffffffffffffffll;
            const long long axx = __double_as_longlong(n.exx) & m;
            const long long ayy = __double_as_longlong(n.eyy) & m;
            const long long axy = __double_as_longlong(n.exy) & m;
            const bool ylt = ayy < axx;
            n.nx = !ylt || axy < ayy;
            n.ny = ylt || axy < axx;
        } else {
            const T axx = fabs(n.exx), ayy = fabs(n.eyy), axy = fabs(n.exy);
            const bool ylt = ayy < axx;
            n.nx = !ylt || axy < ayy;
            n.ny = ylt || axy < axx;
        }
        return n;
    }
    /* take the move: te gains d0t then d1t, ne becomes the move's candidate; written
     * as selects so that the ne chain is add, add, compare, select per step */
    __device__ __forceinline__ void step(const Next &n) {
        using A = Ar<T>;
        const T ta = A::add(te, d0t);
        const T tb = A::add(te, d1t);
        const T tab = A::add(ta, d1t);
        te = n.nx ? (n.ny ? tab : ta) : tb;
        ne = n.nx ? (n.ny ? n.exy : n.exx) : n.eyy;
        cx += n.nx ? sx : 0;
        cy += n.ny ? sy : 0;
    }
};

template <typename IdxT>
__device__ __forceinline__ long long load_idx(const void *idxs, long long i)
{
    return (long long)static_cast<const IdxT *>(idxs)[i];
}

/* warp-aggregated min / max of the frame indices, for the reference's error text */
__device__ __forceinline__ void warp_minmax(long long v, bool valid, DevStatus *st)
{
    long long mn = valid ? v : LLONG_MAX, mx = valid ? v : LLONG_MIN;
    for (int o = 16; o > 0; o >>= 1) {
        mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0 && mn <= mx) {
        atomicMin(&st->idx_min, mn);
        atomicMax(&st->idx_max, mx);
    }
}

template <typename T>
__device__ void write_checkpoints(const LineRec<T> &r, int i, const Coverage<T> &cv,
                                  Checkpoint<T> *__restrict__ cks, DevStatus *st);

/* COUNT_TILES: count the line's (frame, tile) bins (tiles strategy); WALK: also write
 * its walk checkpoints here (lines strategy, which needs no bins) */
/* walks longer than this many columns go to the long-walk list, which
 * walk_ordered_kernel starts first */
constexpr int kLongCols = 96;

/* COUNT_TILES: count the line's (frame, tile) bins (tiles strategy); WALK: also write
 * its walk checkpoints here.  With `longs`, lines longer than kLongCols columns are
 * listed there instead of walked (walk_ordered_kernel walks everything later).  The
 * checkpoint cursor, the long list and the index range take one atomic per block. */
template <typename T, typename IdxT, bool COUNT_TILES, bool WALK>
__global__ void __launch_bounds__(kThreads)
prep_kernel(const T *__restrict__ lines, const void *__restrict__ idxs, long long n_lines,
            long long n_frames, Geometry g, LineRec<T> *__restrict__ recs,
            int *__restrict__ counts, Checkpoint<T> *__restrict__ cks, long long ck_capacity,
            DevStatus *st, int *__restrict__ longs)
{
    __shared__ unsigned long long s_ck[kThreads / 32];
    __shared__ int s_long[kThreads / 32];
    __shared__ long long s_min[kThreads / 32], s_max[kThreads / 32];
    __shared__ unsigned long long s_ck_base, s_long_base;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = i < n_lines;
    long long frame = 0;
    const bool has_idx = idxs != nullptr;
    if (in) frame = has_idx ? load_idx<IdxT>(idxs, i) : (n_frames == 1 ? 0 : i);
    LineRec<T> r;
    r.flags = 0;
    int nck = 0;
    Coverage<T> cv;
    if (in) {
        if (frame < 0 || frame >= n_frames) {
            atomicOr(&st->flags, 1 << CBC_ERR_INDEX);
            atomicMin(&st->bad_line, (unsigned long long)i);
        } else {
            bool too_long = false;
            if (build_rec(lines + 5 * i, r, too_long)) {
                r.frame = (int32_t)frame;
                if (cv.init(r, g)) {
                    r.ncols = cv.lmax - cv.lmin + 1;
                    r.c0 = cv.sa > 0 ? cv.lmin : cv.lmax;
                    nck = (r.ncols + kCkCols - 1) / kCkCols;
                } else {
                    r.flags = 0;        /* walk never enters the frame */
                }
            } else {
                r.flags = 0;
                if (too_long) {
                    atomicOr(&st->flags, 1 << CBC_ERR_RANGE);
                    atomicMin(&st->bad_line, (unsigned long long)i);
                }
            }
        }
    }
    const bool is_long = longs != nullptr && (r.flags & kDrawable) && r.ncols > kLongCols;
    /* warp, then block aggregates */
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = nck;
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    long long mn = (in && has_idx) ? frame : LLONG_MAX, mx = (in && has_idx) ? frame : LLONG_MIN;
    for (int o = 16; o > 0; o >>= 1) {
        mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    const unsigned lm = __ballot_sync(0xffffffffu, is_long);
    if (lane == 31) s_ck[wid] = (unsigned long long)incl;
    if (lane == 0) {
        s_long[wid] = __popc(lm);
        s_min[wid] = mn;
        s_max[wid] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long c = 0;
        int l = 0;
        long long bmn = LLONG_MAX, bmx = LLONG_MIN;
        for (int w = 0; w < kThreads / 32; w++) {
            const unsigned long long tc = s_ck[w];
            s_ck[w] = c;
            c += tc;
            const int tl = s_long[w];
            s_long[w] = l;
            l += tl;
            bmn = min(bmn, s_min[w]);
            bmx = max(bmx, s_max[w]);
        }
        s_ck_base = c ? atomicAdd(&st->cks, c) : 0ull;
        s_long_base = l ? atomicAdd(&st->nlong, (unsigned long long)l) : 0ull;
        if (bmn <= bmx) {
            atomicMin(&st->idx_min, bmn);
            atomicMax(&st->idx_max, bmx);
        }
    }
    __syncthreads();
    if (!in) return;
    if (r.flags & kDrawable) {
        const unsigned long long cb = s_ck_base + s_ck[wid] + (unsigned long long)(incl - nck);
        const bool ck_ok = cb + (unsigned long long)nck <= (unsigned long long)ck_capacity;
        if (!ck_ok) {
            atomicOr(&st->flags, 1 << CBC_ERR_CAPACITY);
            r.ck_base = 0;
        } else {
            r.ck_base = (int32_t)cb;
        }
        if (COUNT_TILES) {
            int *fc = counts + (size_t)frame * g.tiles_x * g.tiles_y;
            for (int ti = cv.lmin / cv.TA; ti <= cv.lmax / cv.TA; ti++) {
                int j0, j1;
                if (!cv.rows(ti, j0, j1)) continue;
                for (int tj = j0; tj <= j1; tj++) atomicAdd(fc + cv.bin(ti, tj, g), 1);
            }
        }
        if (is_long)
            longs[s_long_base + (unsigned long long)(s_long[wid] + __popc(lm & ((1u << lane) - 1u)))] =
                (int)i;
        else if (WALK && ck_ok)
            write_checkpoints(r, (int)i, cv, cks, st);
    }
    recs[i] = r;
}

static __global__ void init_status_kernel(DevStatus *st, int strategy)
{
    st->flags = 0;
    st->strategy = strategy;
    st->bad_line = ~0ull >> 1;
    st->idx_min = LLONG_MAX;
    st->idx_max = LLONG_MIN;
    st->pairs = 0;
    st->cks = 0;
    st->work = 0;
    st->nlong = 0;
}

/* bin offsets: block-local exclusive scan + one atomic per block on the pair cursor */
static __global__ void __launch_bounds__(kThreads)
offsets_kernel(const int *__restrict__ counts, int *__restrict__ offsets,
               int *__restrict__ fillpos, long long n_bins, long long capacity, DevStatus *st)
{
    __shared__ int warp_sums[kThreads / 32];
    __shared__ unsigned long long block_base;
    long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int c = b < n_bins ? counts[b] : 0;
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = c;
    for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int v = lane < kThreads / 32 ? warp_sums[lane] : 0;
        int s = v;
        for (int o = 1; o < 32; o <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += u;
        }
        if (lane < kThreads / 32) warp_sums[lane] = s - v;
        if (lane == kThreads / 32 - 1) block_base = atomicAdd(&st->pairs, (unsigned long long)s);
    }
    __syncthreads();
    if (b >= n_bins) return;
    unsigned long long off = block_base + (unsigned long long)(warp_sums[wid] + incl - c);
    if (c > 0 && off + (unsigned long long)c > (unsigned long long)capacity)
        atomicOr(&st->flags, 1 << CBC_ERR_CAPACITY);
    int o32 = off > (unsigned long long)INT_MAX ? INT_MAX : (int)off;
    offsets[b] = o32;
    fillpos[b] = o32;
}

/* walk line i once and store the iterator state every kCkCols walk columns inside the
 * frame (LineIterator state: position and both errors) */
template <typename T>
__device__ void write_checkpoints(const LineRec<T> &r, int i, const Coverage<T> &cv,
                                  Checkpoint<T> *__restrict__ cks, DevStatus *st)
{
    Walker<T> wk;
    wk.init(r);
    wk.cx = r.x0;
    wk.cy = r.y0;
    wk.te = r.te0;
    wk.ne = r.ne0;
    const int nck = (r.ncols + kCkCols - 1) / kCkCols;
    Checkpoint<T> *ck = cks + r.ck_base;
    int k = 0, next = 0;            /* next checkpoint: the first walk index >= next */
    const int x_end = r.x1, y_end = r.y1, c0 = r.c0, sa = cv.sa, ax = cv.a;
    long long guard = 0;
    /* the walk index starts at or below 0 and grows by at most 1 per step, so a
     * step passes at most one checkpoint */
    while (k < nck && wk.cx != x_end && wk.cy != y_end) {
        const int idx = ((ax ? wk.cy : wk.cx) - c0) * sa;
        if (idx >= next) {
            Checkpoint<T> c;
            c.cx = wk.cx;
            c.cy = wk.cy;
            c.te = wk.te;
            c.ne = wk.ne;
            c.line = i;
            c.seg = k;
            ck[k++] = c;
            next += kCkCols;
        }
        wk.step(wk.decide());
        if (++guard > 4LL * CBC_MAX_WALK + 64) {
            atomicOr(&st->flags, 1 << CBC_ERR_RANGE);
            break;
        }
    }
    for (; k < nck; k++) {
        Checkpoint<T> c;
        c.cx = INT_MIN;
        c.cy = 0;
        c.te = T(0);
        c.ne = T(0);
        c.line = i;
        c.seg = k;
        ck[k] = c;
    }
}

/* tiles strategy: one thread per line writes the line id into each of its bins and
 * then its walk checkpoints */
template <typename T>
__global__ void __launch_bounds__(kThreads)
fill_kernel(const LineRec<T> *__restrict__ recs, long long n_lines, Geometry g,
            int *__restrict__ fillpos, int *__restrict__ pairs, long long capacity,
            Checkpoint<T> *__restrict__ cks, DevStatus *st)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_lines) return;
    if (st->flags & kFatal) return;
    const LineRec<T> r = recs[i];
    if (!(r.flags & kDrawable)) return;
    Coverage<T> cv;
    if (!cv.init(r, g)) return;
    int *fp = fillpos + (size_t)r.frame * g.tiles_x * g.tiles_y;
    for (int ti = cv.lmin / cv.TA; ti <= cv.lmax / cv.TA; ti++) {
        int j0, j1;
        if (!cv.rows(ti, j0, j1)) continue;
        for (int tj = j0; tj <= j1; tj++) {
            int pos = atomicAdd(fp + cv.bin(ti, tj, g), 1);
            if (pos < capacity) pairs[pos] = (int)i;
        }
    }
    write_checkpoints(r, (int)i, cv, cks, st);
}

/* the walks prep_kernel listed as long (thread t < nlong, started first so that the
 * longest sequential walks overlap everything else), then the remaining lines in
 * index order: one thread per line writes its walk checkpoints */
template <typename T>
__global__ void __launch_bounds__(kThreads)
walk_ordered_kernel(const LineRec<T> *__restrict__ recs, long long n_lines,
                    const int *__restrict__ longs, Geometry g, Checkpoint<T> *__restrict__ cks,
                    DevStatus *st)
{
    if (st->flags & kFatal) return;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nlong = (long long)st->nlong;
    long long i = t;
    if (t < nlong) {
        i = longs[t];
    } else {
        i = t - nlong;
        if (i >= n_lines) return;
    }
    const LineRec<T> r = recs[i];
    if (!(r.flags & kDrawable)) return;
    if (t >= nlong && r.ncols > kLongCols) return;       /* walked by the first threads */
    Coverage<T> cv;
    if (!cv.init(r, g)) return;
    write_checkpoints(r, (int)i, cv, cks, st);
}

/* ---- render ---------------------------------------------------------------------- */

template <typename T>
struct Entry {          /* one filled walk position (column) of a line inside the tile */
    int c;              /* long-axis coordinate                                       */
    int sc;             /* short-axis coordinate of the centre pixel                  */
    T te, ne;           /* tangent / normal errors there                              */
};

template <typename T> struct Sentinel;
/* sum: -0 is the only value that no contribution leaves behind (-0 + v = v, and
 * -0 + +0 = +0); max: -inf, below every contribution that can change out */
template <> struct Sentinel<float> {
    static __device__ __forceinline__ float sum() { return -0.0f; }
    static __device__ __forceinline__ bool sum_touched(float v) { return __float_as_uint(v) != 0x80000000u; }
};
template <> struct Sentinel<double> {
    static __device__ __forceinline__ double sum() { return -0.0; }
    static __device__ __forceinline__ bool sum_touched(double v) {
        return (unsigned long long)__double_as_longlong(v) != 0x8000000000000000ull;
    }
};

template <typename T>
__device__ __forceinline__ void combine_max(T *addr, T v);

template <>
__device__ __forceinline__ void combine_max<float>(float *addr, float v)
{
    /* acc = std::max(acc, v): replace only when acc < v (bresenham.cpp:71) */
    unsigned *ua = reinterpret_cast<unsigned *>(addr);
    unsigned old = *reinterpret_cast<volatile unsigned *>(ua);
    while (__uint_as_float(old) < v) {
        unsigned prev = atomicCAS(ua, old, __float_as_uint(v));
        if (prev == old) break;
        old = prev;
    }
}

template <>
__device__ __forceinline__ void combine_max<double>(double *addr, double v)
{
    unsigned long long *ua = reinterpret_cast<unsigned long long *>(addr);
    unsigned long long old = *reinterpret_cast<volatile unsigned long long *>(ua);
    while (__longlong_as_double((long long)old) < v) {
        unsigned long long prev = atomicCAS(ua, old, (unsigned long long)__double_as_longlong(v));
        if (prev == old) break;
        old = prev;
    }
}

/* window [jlo, jhi] of short-axis offsets from the centre that the span can reach:
 * ne moves by ns per step, the span stops once |ne| >= ne_thr (float estimate, one
 * pixel of margin each side), clipped to the frame / tile range [s_lo, s_hi] */
template <typename T>
__device__ __forceinline__ int span_window(const SlotParams<T> &p, int sc, T ne, int s_lo,
                                           int s_hi, int &jlo)
{
    const float R = (float)p.ne_thr * fabsf(p.rns);
    const float u = (float)ne * p.rns;
    const float up = R - u, dn = R + u;
    const int kp = up < 2e9f ? (int)floorf(up) + 1 : INT_MAX / 4;
    const int km = dn < 2e9f ? (int)floorf(dn) + 1 : INT_MAX / 4;
    jlo = max(-max(km, 0), s_lo - sc);
    const int jhi = min(max(kp, 0), s_hi - sc);
    return max(0, jhi - jlo + 1);
}

template <typename T>
__device__ __forceinline__ void global_combine_max(T *addr, T v);

template <>
__device__ __forceinline__ void global_combine_max<float>(float *addr, float v)
{
    if (v > 0.0f) {
        /* positive v: the integer order of the bit patterns is std::max's order for
         * every out except a negative-signed NaN */
        atomicMax(reinterpret_cast<int *>(addr), __float_as_int(v));
    } else if (v == v) {
        combine_max(addr, v);
    }
}

template <>
__device__ __forceinline__ void global_combine_max<double>(double *addr, double v)
{
    if (v > 0.0) {
        atomicMax(reinterpret_cast<long long *>(addr), __double_as_longlong(v));
    } else if (v == v) {
        combine_max(addr, v);
    }
}

/* ---- lines-strategy pixel enumeration ---------------------------------------------
 * Work items are (line, kSeg-column segment) pairs, kItemsPerCk per walk checkpoint.
 * A warp takes 32 of them from an atomic counter, one per lane, resumes every lane's
 * walk (bresenham.hpp:352-383 outer loop) from its checkpoint (walking past the columns
 * before the segment) and handles the segment's columns in kSeg rounds, one column
 * per lane and round:
 *   spans:   level k = 0, 1, 2, ... of all 32 columns at once: every lane advances
 *            the two span walks of its column (the inner loops, :369-380) by one step
 *            with the reference's float increments, and the visited in-frame pixels
 *            of the level go into per-warp rings in shared memory (ballot +
 *            popcount give the positions);
 *   pixels:  whenever a ring holds 32 pixels, every lane takes one, evaluates the
 *            error E with the reference's rounding and, for E <= 1, calls
 *                act.pixel(slots, slot, x, y, E, te, ne, pre)
 *            where pre = act.prefetch(slots, slot, x, y) was issued before the
 *            error arithmetic (the action's global loads for the pixel).
 * A span walk ends at its first step with |ne| >= threshold (the reference's loop
 * condition) or when it leaves the frame.  The walks stay sequential per lane, as in
 * the reference, while the expensive per-pixel work runs on full warps.
 * act.item_begin(lane, slots) / act.item_end(lane, slots) bracket each warp item; an action
 * that needs no error (and is handed every visited pixel) clears kNeedsError.  The
 * forward, the max-overlap winner pass and the adjoint are such actions. */

constexpr int kSegWarps = 4;
constexpr int kSegMinBlocks = 6;   /* resident CTAs per SM the register budget targets */
constexpr int kRing = 128;         /* slots per ring, a power of two >= 31 + 64 */

template <typename T>
struct DriveArgs {
    const LineRec<T> *recs;
    const Checkpoint<T> *cks;
    int H, W;
    DevStatus *st;
    unsigned long long *work;      /* work-item counter, zeroed before the launch */
};

/* what the error evaluation reads per slot: one 16-byte load for float */
template <typename T>
struct alignas(16) EvalSlot {
    T len, rlen, ww, rww;
};

/* per-slot (lane) data of a warp's current items, one array per field so that 32
 * lanes reading 32 different slots hit distinct shared-memory banks */
template <typename T>
struct SlotTable {
    EvalSlot<T> ev[32];
    T len2[32];
    int fast[32];        /* len and ww in the range of the reciprocal division */
    long long fbase[32]; /* frame * H * W                                      */
    int line[32];        /* line index, -1 for an empty slot                   */
};

/* a visited pixel waiting for evaluation: walk errors and frame coordinates, one
 * 16-byte shared-memory access for float */
template <typename T>
struct alignas(16) RingPixel {
    T te, ne;
    int x, y;
};

template <typename T>
struct PixelRing {
    RingPixel<T> px[kRing];
    unsigned char slot[kRing];     /* owner lane of each pixel */
};

/* Comparisons of the segment driver.  For double they compare bit patterns on the
 * integer pipe (the float64 render is bound by the FP64 pipe): for doubles that are
 * not NaN the signed order of the patterns of non-negative values is their order, and
 * a negative pattern is a negative value or -0.  The walk's errors, the span
 * threshold (>= 0) and the pixel errors (>= 0) are never NaN. */
template <typename T>
__device__ __forceinline__ bool abs_lt(T v, T thr) { return fabs(v) < thr; }
template <>
__device__ __forceinline__ bool abs_lt<double>(double v, double thr)
{
    return (__double_as_longlong(v) & 0x7fffffffffffffffll) < __double_as_longlong(thr);
}

/* t < 0 || t > hi, for hi >= 0 */
template <typename T>
__device__ __forceinline__ bool outside(T t, T hi) { return t < T(0) || t > hi; }
template <>
__device__ __forceinline__ bool outside<double>(double t, double hi)
{
    const long long b = __double_as_longlong(t);
    return (b < 0 && b != LLONG_MIN) || b > __double_as_longlong(hi);
}

/* E <= 1 for an error E >= 0 */
template <typename T>
__device__ __forceinline__ bool le_one(T e) { return e <= T(1); }
template <>
__device__ __forceinline__ bool le_one<double>(double e)
{
    return __double_as_longlong(e) <= 0x3ff0000000000000ll;
}

/* an end-cap pixel (te < 0 or te > len^2) whose error is surely above 1: the error
 * E = (ta^2 + ne^2) / (len^2 w^2) in exact arithmetic, with ta = max(-te, te - len^2),
 * and the reference's float evaluation of E is within a few ulp of it, so
 * ta^2 + ne^2 > len^2 w^2 (1 + 2^-13) in any rounding means E > 1: the pixel is not
 * drawn and need not be queued.  Inside pixels are not tested: the span condition
 * already bounds their error by 1. */
template <typename T>
__device__ __forceinline__ bool cap_far(T te, T ne, T len2, T lim)
{
    if constexpr (sizeof(T) == sizeof(double)) {
        return false;   /* four FP64 operations per span step cost the float64 render more */
    } else {
        const T ta = fmax(-te, te - len2);
        return ta * ta + ne * ne > lim;
    }
}

/* actions that draw only some lines define keep_line(line) */
template <class A, class = void> struct FiltersLines : std::false_type {};
template <class A>
struct FiltersLines<A, std::void_t<decltype(&A::keep_line)>> : std::true_type {};

/* actions that combine a drain batch's results across the warp define batch_end(lane),
 * called by all 32 lanes after every batch */
template <class A, class = void> struct EndsBatches : std::false_type {};
template <class A>
struct EndsBatches<A, std::void_t<decltype(&A::batch_end)>> : std::true_type {};

template <typename T, class Act>
__device__ __forceinline__ void drive_segments(const DriveArgs<T> &a, Act &act)
{
    using A = Ar<T>;
    __shared__ SlotTable<T> slot_s[kSegWarps];
    __shared__ PixelRing<T> ring_s[kSegWarps][2];
    if (a.st->flags & kFatal) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    SlotTable<T> &S = slot_s[warp];
    PixelRing<T> *rg = ring_s[warp];
    const long long total = (long long)a.st->cks * kItemsPerCk;
    const unsigned lanes_below = (1u << lane) - 1u;
    /* ring cursors, equal in every lane: ring 0 holds pixels within the segment's
     * extent along the line (0 <= te <= len^2, where the error is the normal term
     * alone), ring 1 the end-cap pixels, whose error takes the longer exact path;
     * separate rings keep every evaluation round on one path */
    unsigned head0 = 0, tail0 = 0, head1 = 0, tail1 = 0;

    auto store = [&](bool cap, unsigned q, T te, T ne, int x, int y) {
        PixelRing<T> &R = rg[cap ? 1 : 0];
        RingPixel<T> v;
        v.te = te;
        v.ne = ne;
        v.x = x;
        v.y = y;
        R.px[q & (kRing - 1)] = v;
        R.slot[q & (kRing - 1)] = (unsigned char)lane;
    };
    /* append the lanes' pixels with `take` set */
    auto push = [&](bool take, bool cap, T te, T ne, int x, int y) {
        const unsigned m1 = __ballot_sync(0xffffffffu, take && cap);
        const unsigned m0 = __ballot_sync(0xffffffffu, take && !cap);
        if (take)
            store(cap, cap ? tail1 + __popc(m1 & lanes_below) : tail0 + __popc(m0 & lanes_below),
                  te, ne, x, y);
        tail0 += __popc(m0);
        tail1 += __popc(m1);
    };
    /* the same for two pixels per lane: all (a) pixels precede all (b) pixels */
    auto push2 = [&](bool ta, bool ca, T tea, T nea, int xa, int ya,
                     bool tb, bool cb, T teb, T neb, int xb, int yb) {
        const unsigned a1 = __ballot_sync(0xffffffffu, ta && ca);
        const unsigned a0 = __ballot_sync(0xffffffffu, ta && !ca);
        const unsigned b1 = __ballot_sync(0xffffffffu, tb && cb);
        const unsigned b0 = __ballot_sync(0xffffffffu, tb && !cb);
        const unsigned na1 = __popc(a1), na0 = __popc(a0);
        if (ta)
            store(ca, ca ? tail1 + __popc(a1 & lanes_below) : tail0 + __popc(a0 & lanes_below),
                  tea, nea, xa, ya);
        if (tb)
            store(cb, cb ? tail1 + na1 + __popc(b1 & lanes_below)
                         : tail0 + na0 + __popc(b0 & lanes_below),
                  teb, neb, xb, yb);
        tail0 += na0 + __popc(b0);
        tail1 += na1 + __popc(b1);
    };
    /* evaluate ring pixels, 32 at a time, until at most `keep` remain in the ring */
    auto drain_ring = [&](PixelRing<T> &R, unsigned &head, unsigned tail, unsigned keep,
                          bool cap) {
        while (tail - head > keep) {
            __syncwarp();
            const unsigned n = min(tail - head, 32u);
            if ((unsigned)lane < n) {
                const unsigned q = (head + lane) & (kRing - 1);
                const int slot = R.slot[q];
                const RingPixel<T> v = R.px[q];
                /* the action's own loads first: they complete under the error arithmetic */
                const typename Act::Pre pre = act.prefetch(S, slot, v.x, v.y);
                if constexpr (Act::kNeedsError) {
                    const EvalSlot<T> ev = S.ev[slot];
                    SlotParams<T> p;
                    p.len = ev.len;
                    p.rlen = ev.rlen;
                    p.ww = ev.ww;
                    p.rww = ev.rww;
                    p.fast = S.fast[slot];
                    if (cap) p.len2 = S.len2[slot];
                    const T nf = A::nterm(v.ne, p);
                    const T E = cap ? A::error(v.te, nf, p) : A::error_inside(nf, p);
                    if (le_one(E)) act.pixel(S, slot, v.x, v.y, E, v.te, v.ne, pre);
                } else {
                    /* the action decides from its own data which visited pixels count
                     * (the max-overlap adjoint: the pixel's winner) */
                    act.pixel(S, slot, v.x, v.y, T(0), v.te, v.ne, pre);
                }
            }
            if constexpr (EndsBatches<Act>::value) act.batch_end(lane);
            head += n;
            __syncwarp();
        }
    };
    auto drain = [&](unsigned keep) {
        drain_ring(rg[0], head0, tail0, keep, false);
        drain_ring(rg[1], head1, tail1, keep, true);
    };

    for (;;) {
        long long base = 0;
        if (lane == 0) base = (long long)atomicAdd(a.work, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total) break;
        const long long item = base + lane;
        S.line[lane] = -1;

        Walker<T> wk;
        int x_end = 0, y_end = 0, c0 = 0, sa = 1, lo = 0, hi = -1, ax = 0, s_hi = -1;
        T ts = T(0), ns = T(0), thr = T(0), len2 = T(0), cap_lim = T(0);
        bool cols = false;             /* columns of this item left to find */
        if (item < total) {
            const Checkpoint<T> ck = a.cks[item / kItemsPerCk];
            bool keep = true;
            if constexpr (FiltersLines<Act>::value) keep = act.keep_line(ck.line);
            if (ck.cx != INT_MIN && keep) {
                const LineRec<T> r = a.recs[ck.line];
                ax = r.flags & kAxisY;
                wk.init(r);
                wk.cx = ck.cx;
                wk.cy = ck.cy;
                wk.te = ck.te;
                wk.ne = ck.ne;
                x_end = r.x1;
                y_end = r.y1;
                c0 = r.c0;
                sa = ax ? wk.sy : wk.sx;
                lo = ck.seg * kCkCols + (int)(item % kItemsPerCk) * kSeg;
                hi = min(lo + kSeg - 1, r.ncols - 1);
                s_hi = (ax ? a.W : a.H) - 1;
                ts = ax ? r.t0 : r.t1;
                ns = ax ? r.t1 : -r.t0;
                thr = r.ne_thr;
                len2 = r.len2;
                cap_lim = r.len2 * r.ww * T(1.0 + 0x1p-13);
                EvalSlot<T> ev;
                ev.len = r.len;
                ev.rlen = r.rlen;
                ev.ww = r.ww;
                ev.rww = r.rww;
                S.ev[lane] = ev;
                S.len2[lane] = r.len2;
                S.fast[lane] = (r.flags & kFastDiv) ? 1 : 0;
                S.fbase[lane] = (long long)r.frame * a.H * a.W;
                cols = lo <= hi;                 /* a last item past the walk's end is empty */
                S.line[lane] = cols ? ck.line : -1;
            }
        }
        act.item_begin(lane, S);
        __syncwarp();

        int guard = 0;
        #pragma unroll 1
        for (int b = 0; b < kSeg && __any_sync(0xffffffffu, cols); b++) {
            /* this lane's next column: the position of the next long-axis step with
             * walk index in [lo, hi] */
            bool col = false;
            int c = 0, sc = 0;
            T te_c = T(0), ne_c = T(0);
            while (cols && wk.cx != x_end && wk.cy != y_end) {
                const typename Walker<T>::Next mv = wk.decide();
                const int cc = ax ? wk.cy : wk.cx;
                const int idx = (cc - c0) * sa;
                if (idx > hi) break;
                const bool here = (ax ? mv.ny : mv.nx) && idx >= lo;
                if (here) {
                    col = true;
                    c = cc;
                    sc = ax ? wk.cx : wk.cy;
                    te_c = wk.te;
                    ne_c = wk.ne;
                    if (idx == hi) cols = false;
                }
                wk.step(mv);
                if (++guard > 4 * CBC_MAX_WALK + 64) {
                    atomicOr(&a.st->flags, 1 << CBC_ERR_RANGE);
                    col = false;
                    break;
                }
                if (here) break;
            }
            if (!col) cols = false;

            /* level 0: the column's centre pixel */
            const bool cap_c = outside(te_c, len2);
            push(col && sc >= 0 && sc <= s_hi && !(cap_c && cap_far(te_c, ne_c, len2, cap_lim)),
                 cap_c, te_c, ne_c, ax ? sc : c, ax ? c : sc);
            drain(31);
            /* levels 1, 2, ...: one step of the upward and the downward span walk */
            T tu = te_c, nu = ne_c, td = te_c, nd = ne_c;
            bool up = col, dn = col;
            for (int k = 1;; k++) {
                /* both walks step every level; a finished walk's values go unused */
                tu = A::add(tu, ts);
                nu = A::add(nu, ns);
                td = A::sub(td, ts);
                nd = A::sub(nd, ns);
                const int su = sc + k, sd = sc - k;
                up = up && abs_lt(nu, thr) && su <= s_hi;
                dn = dn && abs_lt(nd, thr) && sd >= 0;
                if (!__any_sync(0xffffffffu, up || dn)) break;
                const bool cap_u = outside(tu, len2), cap_d = outside(td, len2);
                push2(up && su >= 0 && !(cap_u && cap_far(tu, nu, len2, cap_lim)), cap_u, tu, nu,
                      ax ? su : c, ax ? c : su,
                      dn && sd <= s_hi && !(cap_d && cap_far(td, nd, len2, cap_lim)), cap_d, td,
                      nd, ax ? sd : c, ax ? c : sd);
                drain(31);
            }
        }
        drain(0);
        __syncwarp();
        act.item_end(lane, S);
        __syncwarp();
    }
}

/* the float gaussian's table copied into shared memory at kernel start (random
 * per-lane entries: a shared-memory gather instead of one L1 sector per lane);
 * null for the other profiles and for double.  Every thread of the CTA calls it. */
template <typename T, int K>
__device__ __forceinline__ const float *stage_gauss_table()
{
    if constexpr (K == CBC_GAUSSIAN && sizeof(T) == sizeof(float)) {
        __shared__ float2 tab[CBC_EXP_TABLE_N];
        const float2 *src = reinterpret_cast<const float2 *>(&cbc_gauss_table[0][0]);
        for (int i = threadIdx.x; i < CBC_EXP_TABLE_N; i += blockDim.x) tab[i] = src[i];
        __syncthreads();
        return reinterpret_cast<const float *>(tab);
    } else {
        return nullptr;
    }
}

/* grid of a persistent kernel: the CTAs of `threads` threads that are resident at
 * once on the current device (cached per kernel and device) */
template <typename F>
unsigned resident_grid(F kernel, int threads)
{
    static std::atomic<int> cache[64];
    int dev = 0;
    cudaGetDevice(&dev);
    std::atomic<int> &c = cache[dev & 63];
    int g = c.load(std::memory_order_relaxed);
    if (g == 0) {
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
        g = (sms > 0 ? sms : 132) * (per_sm > 0 ? per_sm : 1);
        c.store(g, std::memory_order_relaxed);
    }
    return (unsigned)g;
}

/* ---- adjoint helpers shared by the 2-D and 3-D gradients ----------------------------
 * A line draws v = max_val K(d / w), d the distance from the pixel (voxel) centre to the
 * segment.  With q the nearest point of the segment and s its position along it, the
 * envelope theorem gives dv/dp0 = kappa (1 - s)(q - P), dv/dp1 = kappa s (q - P) and
 * dv/dw = -kappa d^2 / w with kappa = max_val K'(d / w) / (w d), which is finite at
 * d = 0 for the smooth profiles.  kappa as a function of d^2: k0 + k1 d^2 (biweight,
 * parabolic with k1 = 0), k0 exp(k1 d^2) (gaussian), k0 / d (triangular, 0 at d = 0),
 * 0 (rectangular); rw = 1 / w.  Profiles of include.hpp:447-468. */
template <typename T, int K>
__device__ __forceinline__ void kappa_consts(T w, T max_val, T &k0, T &k1, T &rw)
{
    rw = T(1) / w;
    const T rww = rw * rw;
    switch (K) {
    case CBC_BIWEIGHT:
        k0 = T(-3.75) * max_val * rww;
        k1 = -k0 * rww;
        break;
    case CBC_GAUSSIAN:
        k0 = T(-9) * T(CBC_GAUSS_C) * max_val * rww;
        k1 = T(-4.5) * rww;
        break;
    case CBC_PARABOLIC:
        k0 = T(-1.5) * max_val * rww;
        k1 = T(0);
        break;
    case CBC_RECTANGULAR:
        k0 = k1 = T(0);
        break;
    default:
        k0 = -max_val * rw;
        k1 = T(0);
        break;
    }
}

template <typename T, int K>
__device__ __forceinline__ T kappa_d2(T d2, T k0, T k1)
{
    switch (K) {
    case CBC_BIWEIGHT:  return k0 + k1 * d2;
    case CBC_GAUSSIAN:  return k0 * exp(k1 * d2);
    case CBC_PARABOLIC: return k0;
    case CBC_RECTANGULAR: return T(0);
    default: {
        const T d = sqrt(d2);
        return d > T(0) ? k0 / d : T(0);
    }
    }
}

template <typename T> __device__ __forceinline__ T fma_rn(T a, T b, T c);
template <> __device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <> __device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

/* p q - r s within 2 ulp: the product r s and its FMA error term (Kahan's difference
 * of products) */
template <typename T>
__device__ __forceinline__ T diff_of_products(T p, T q, T r, T s)
{
    const T rs = r * s;
    return fma_rn(p, q, -rs) + fma_rn(-r, s, rs);
}

/* host-side error reporting, defined in cbc_draw_lines.cu */
int fail(int code, const std::string &msg);
/* offsets of the line records and walk checkpoints in a draw_lines workspace laid out
 * for these sizes and tuning (false for an invalid tuning), defined in cbc_draw_lines.cu */
bool draw_workspace_parts(long long n_frames, long long H, long long W, long long n_lines,
                          long long capacity, long long ck_capacity, size_t elem,
                          const cbc_tuning *tuning, size_t *recs, size_t *cks);
void clear_error();
/* adds n to the library's kernel-launch counter (reported by cbc_profile_read) */
void note_launches(int n);

}  // namespace cbc

#endif /* CBC_COMMON_CUH */
