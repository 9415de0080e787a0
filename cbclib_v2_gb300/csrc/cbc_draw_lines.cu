/*
 * cbc_draw_lines.cu — GB300 (sm_103a) thick-line rasteriser behind the C ABI of
 * include/cbc_draw_lines.h.
 *
 * Semantics: those of the reference CPU path (cbclib_v2/_src/src/bresenham.cpp:38-101
 * with the walk of bresenham.hpp:233-383): every line is walked with the reference's
 * incremental Bresenham errors, each visited pixel with error <= 1 receives
 * max_val * K(sqrt(error)), combined into `out` by sum or max.  All float arithmetic
 * is spelled with round-to-nearest intrinsics and the file is built with
 * --fmad=false, so every rounding matches the reference; the reference's
 * double-rounded steps go through exact.cuh.
 *
 * Pipeline (one stream, no host synchronisation):
 *   1. prep_kernel   one thread per line: frame index check, walk parameters
 *                    (LineRec), conservative tile coverage -> per-bin counts.
 *   2. offsets_kernel  block scan of the per-bin counts, one atomic per block ->
 *                    bin offsets into the pair buffer (a counting sort on the
 *                    (frame, tile) key), capacity check.
 *   3. fill_kernel   one thread per line: line id into each of its bins.
 *   4. render_kernel one CTA per (frame, tile) bin with lines: stage the output tile
 *                    in shared memory, replay each line's walk to the tile's columns
 *                    (one thread per line), then evaluate the spans of all
 *                    (line, column) entries in parallel with shared-memory atomics,
 *                    write the tile back once.  Empty bins are never touched.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <limits.h>
#include <stdio.h>
#include <string.h>
#include <string>
#include <mutex>
#include <vector>

#include "cbc_draw_lines.h"
#include "exact.cuh"

#define CBC_VERSION "cbclib_v2_gb300 0.1.0 (sm_103a)"

namespace cbc {

constexpr int kThreads = 256;
constexpr int kMaxChunk = 32;
constexpr int kDefaultTileW = 64;
constexpr int kDefaultTileH = 64;
constexpr int kDefaultChunk = 16;
constexpr int kFatal = (1 << CBC_ERR_INDEX) | (1 << CBC_ERR_CAPACITY) | (1 << CBC_ERR_RANGE);
constexpr int kInvalidEntry = INT_MIN;

/* ---- per-line walk record ------------------------------------------------------ */

enum : int { kAxisY = 1, kStepXNeg = 2, kStepYNeg = 4, kDrawable = 8 };

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
    int32_t frame, flags;
};

/* status block at the start of the workspace */
struct DevStatus {
    int flags;
    int reserved;
    unsigned long long bad_line;
    long long idx_min;
    long long idx_max;
    unsigned long long pairs;      /* running pair cursor == pairs_needed */
};

/* ---- arithmetic in the reference's rounding ----------------------------------- */

template <typename T> struct Ar;

template <> struct Ar<float> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt(float a) { return __fsqrt_rn(a); }
    static __device__ __forceinline__ float from_int(int v) { return __int2float_rn(v); }
    static __device__ __forceinline__ float normal_term(float ne, float len) {
        return cbc_normal_term(ne, len);
    }
    static __device__ __forceinline__ float error(float te, float nf, float len, float len2,
                                                  float ww) {
        return cbc_pixel_error(te, nf, len, len2, ww);
    }
    template <int K>
    static __device__ __forceinline__ float profile(float x) { return cbc_profile_f32(K, x); }
};

template <> struct Ar<double> {
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ double sqrt(double a) { return __dsqrt_rn(a); }
    static __device__ __forceinline__ double from_int(int v) { return (double)v; }
    /* normal_error: T accumulator fed with pow(b, 2) = fl(b * b) (bresenham.hpp:284-289) */
    static __device__ __forceinline__ double normal_term(double ne, double len) {
        double b = __ddiv_rn(ne, len);
        return __dmul_rn(b, b);
    }
    /* error(): fl(fl(fl(a * a) + nf) / ww) (bresenham.hpp:291-296) */
    static __device__ __forceinline__ double error(double te, double nf, double len,
                                                   double len2, double ww) {
        double m1 = -te, m2 = __dsub_rn(te, len2);
        double ta = (m1 < m2) ? m2 : m1;
        if (ta < 0.0) ta = 0.0;
        double a = __ddiv_rn(ta, len);
        return __ddiv_rn(__dadd_rn(__dmul_rn(a, a), nf), ww);
    }
    template <int K>
    static __device__ __forceinline__ double profile(double x) { return cbc_profile_f64(K, x); }
};

/* ---- line preparation ---------------------------------------------------------- */

template <typename T>
__device__ __forceinline__ bool finite_val(T v) { return isfinite(v); }

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
    r.flags = axis | (sx < 0 ? kStepXNeg : 0) | (sy < 0 ? kStepYNeg : 0) | kDrawable;
    return true;
}

struct Geometry {
    int H, W;
    int tile_w, tile_h;
    int tiles_x, tiles_y;
};

/* Conservative set of tiles holding the pixels the walk can draw: the walk covers the
 * long-axis range [m_pt0, m_pt1) exactly; at long coordinate c its centre pixel lies
 * within 1 px of the line and its spans stop where |normal distance| >= width, i.e.
 * within width * len / |t_long| of the line along the short axis. */
template <typename T, typename Fn>
__device__ void for_each_tile(const LineRec<T> &r, const Geometry &g, Fn fn)
{
    const int a = r.flags & kAxisY;
    const int sxs = (r.flags & kStepXNeg) ? -1 : 1, sys = (r.flags & kStepYNeg) ? -1 : 1;
    const int sa = a ? sys : sxs;
    int first = a ? r.y0 : r.x0;
    int last = (a ? r.y1 : r.x1) - sa;
    int lmin = min(first, last), lmax = max(first, last);
    const int ext_a = a ? g.H : g.W, ext_s = a ? g.W : g.H;
    const int TA = a ? g.tile_h : g.tile_w, TS = a ? g.tile_w : g.tile_h;
    lmin = max(lmin, 0);
    lmax = min(lmax, ext_a - 1);
    if (lmin > lmax) return;
    const float ta = (float)(a ? r.t1 : r.t0), ts = (float)(a ? r.t0 : r.t1);
    const float pa = (float)(a ? r.py : r.px), ps = (float)(a ? r.px : r.py);
    const float slope = ts / ta;
    const float hw = (float)r.w * (float)r.len / fabsf(ta) + 2.0f;
    for (int ti = lmin / TA; ti <= lmax / TA; ti++) {
        int ca = max(lmin, ti * TA), cb = min(lmax, ti * TA + TA - 1);
        float s0 = ps + ((float)ca - pa) * slope, s1 = ps + ((float)cb - pa) * slope;
        float smin = fminf(s0, s1) - hw, smax = fmaxf(s0, s1) + hw;
        if (!(smax >= 0.0f) || !(smin <= (float)(ext_s - 1))) continue;
        int j0 = max(0, (int)floorf(fmaxf(smin, -1.0f))) / TS;
        int j1 = min(ext_s - 1, (int)floorf(fminf(smax, (float)ext_s))) / TS;
        for (int tj = j0; tj <= j1; tj++) fn(a ? (ti * g.tiles_x + tj) : (tj * g.tiles_x + ti));
    }
}

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

template <typename T, typename IdxT>
__global__ void __launch_bounds__(kThreads)
prep_kernel(const T *__restrict__ lines, const void *__restrict__ idxs, long long n_lines,
            long long n_frames, Geometry g, LineRec<T> *__restrict__ recs,
            int *__restrict__ counts, DevStatus *st)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool in = i < n_lines;
    long long frame = 0;
    bool has_idx = idxs != nullptr;
    if (in) frame = has_idx ? load_idx<IdxT>(idxs, i) : (n_frames == 1 ? 0 : i);
    if (has_idx) warp_minmax(frame, in, st);
    if (!in) return;
    LineRec<T> r;
    r.flags = 0;
    if (frame < 0 || frame >= n_frames) {
        atomicOr(&st->flags, 1 << CBC_ERR_INDEX);
        atomicMin(&st->bad_line, (unsigned long long)i);
        recs[i] = r;
        return;
    }
    bool too_long = false;
    if (build_rec(lines + 5 * i, r, too_long)) {
        r.frame = (int32_t)frame;
        int *fc = counts + (size_t)frame * g.tiles_x * g.tiles_y;
        for_each_tile(r, g, [&](int b) { atomicAdd(fc + b, 1); });
    } else {
        r.flags = 0;
        if (too_long) {
            atomicOr(&st->flags, 1 << CBC_ERR_RANGE);
            atomicMin(&st->bad_line, (unsigned long long)i);
        }
    }
    recs[i] = r;
}

__global__ void init_status_kernel(DevStatus *st)
{
    st->flags = 0;
    st->reserved = 0;
    st->bad_line = ~0ull >> 1;
    st->idx_min = LLONG_MAX;
    st->idx_max = LLONG_MIN;
    st->pairs = 0;
}

/* bin offsets: block-local exclusive scan + one atomic per block on the pair cursor */
__global__ void __launch_bounds__(kThreads)
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

template <typename T>
__global__ void __launch_bounds__(kThreads)
fill_kernel(const LineRec<T> *__restrict__ recs, long long n_lines, Geometry g,
            int *__restrict__ fillpos, int *__restrict__ pairs, long long capacity,
            const DevStatus *st)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_lines) return;
    if (st->flags & kFatal) return;
    LineRec<T> r = recs[i];
    if (!(r.flags & kDrawable)) return;
    int *fp = fillpos + (size_t)r.frame * g.tiles_x * g.tiles_y;
    for_each_tile(r, g, [&](int b) {
        int pos = atomicAdd(fp + b, 1);
        if (pos < capacity) pairs[pos] = (int)i;
    });
}

/* ---- render ---------------------------------------------------------------------- */

template <typename T>
struct Entry {          /* one filled walk position (column) of a line inside the tile */
    int c;              /* long-axis coordinate                                       */
    int sc;             /* short-axis coordinate of the centre pixel                  */
    T te, ne;           /* tangent / normal errors there                              */
};

template <typename T>
struct SlotParams {     /* per line of the current chunk */
    T ts, ns;           /* tangent / normal derivative along the short axis           */
    T len, len2, ww;
    int ss;             /* step sign along the short axis (first span half)            */
    int axis;
};

template <typename T>
__device__ __forceinline__ void combine_max(T *addr, T v);

template <>
__device__ __forceinline__ void combine_max<float>(float *addr, float v)
{
    /* out = std::max(out, v): replace only when out < v (bresenham.cpp:71) */
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

template <typename T>
struct RenderArgs {
    T *out;
    const LineRec<T> *recs;
    const int *counts;
    const int *offsets;
    const int *pairs;
    DevStatus *st;
    Geometry g;
    T max_val;
    int chunk;
    int ent_cap;
};

template <typename T>
__host__ __device__ constexpr size_t render_smem_bytes(int tile_w, int tile_h, int ent_cap)
{
    return (size_t)tile_w * tile_h * sizeof(T) + (size_t)ent_cap * sizeof(Entry<T>) +
           (size_t)ent_cap + kMaxChunk * sizeof(SlotParams<T>) + (kMaxChunk + 1) * sizeof(int) +
           64;
}

template <typename T, int K, int OV>
__global__ void __launch_bounds__(kThreads)
render_kernel(RenderArgs<T> a)
{
    using A = Ar<T>;
    extern __shared__ __align__(16) unsigned char smem[];
    const int bin = blockIdx.x;
    const int cnt = a.counts[bin];
    if (cnt == 0) return;
    if (a.st->flags & kFatal) return;

    const Geometry &g = a.g;
    const int tpf = g.tiles_x * g.tiles_y;
    const int frame = bin / tpf;
    const int t = bin - frame * tpf;
    const int ty = t / g.tiles_x, tx = t - ty * g.tiles_x;
    const int x0 = tx * g.tile_w, y0 = ty * g.tile_h;
    const int tw = min(g.tile_w, g.W - x0), th = min(g.tile_h, g.H - y0);

    T *tile = reinterpret_cast<T *>(smem);
    Entry<T> *ent = reinterpret_cast<Entry<T> *>(tile + (size_t)g.tile_w * g.tile_h);
    SlotParams<T> *prm = reinterpret_cast<SlotParams<T> *>(ent + a.ent_cap);
    int *base = reinterpret_cast<int *>(prm + kMaxChunk);
    unsigned char *eslot = reinterpret_cast<unsigned char *>(base + kMaxChunk + 1);

    T *gout = a.out + ((size_t)frame * g.H + y0) * g.W + x0;
    for (int e = threadIdx.x; e < tw * th; e += kThreads) {
        int r = e / tw, c = e - r * tw;
        tile[e] = gout[(size_t)r * g.W + c];
    }

    const int *seg = a.pairs + a.offsets[bin];
    for (int cb = 0; cb < cnt; cb += a.chunk) {
        const int n = min(a.chunk, cnt - cb);
        /* phase A: per-line slot parameters and the count of in-tile walk columns */
        int my_count = 0, c_begin = 0, c_lo = 0, c_hi = -1, sa = 1;
        LineRec<T> r;
        if (threadIdx.x < n) {
            r = a.recs[seg[cb + threadIdx.x]];
            const int ax = r.flags & kAxisY;
            const int sx = (r.flags & kStepXNeg) ? -1 : 1, sy = (r.flags & kStepYNeg) ? -1 : 1;
            sa = ax ? sy : sx;
            const int la0 = ax ? y0 : x0, la1 = ax ? y0 + th - 1 : x0 + tw - 1;
            const int first = ax ? r.y0 : r.x0, last = (ax ? r.y1 : r.x1) - sa;
            if (sa > 0) { c_lo = max(first, la0); c_hi = min(last, la1); c_begin = c_lo; }
            else        { c_lo = max(last, la0);  c_hi = min(first, la1); c_begin = c_hi; }
            my_count = max(0, c_hi - c_lo + 1);
            SlotParams<T> p;
            p.ts = ax ? r.t0 : r.t1;              /* d te / d short */
            p.ns = ax ? r.t1 : -r.t0;             /* d ne / d short: normal = (t1, -t0) */
            p.len = r.len;
            p.len2 = r.len2;
            p.ww = r.ww;
            p.ss = ax ? sx : sy;
            p.axis = ax;
            prm[threadIdx.x] = p;
        }
        /* exclusive scan of the counts over the chunk (n <= 32: warp 0) */
        if (threadIdx.x < 32) {
            int v = threadIdx.x < n ? my_count : 0, s = v;
            for (int o = 1; o < 32; o <<= 1) {
                int u = __shfl_up_sync(0xffffffffu, s, o);
                if ((int)threadIdx.x >= o) s += u;
            }
            base[threadIdx.x] = s - v;
            if (threadIdx.x == 31) base[kMaxChunk] = s;
        }
        __syncthreads();
        const int total = base[kMaxChunk];
        for (int e = threadIdx.x; e < total; e += kThreads) ent[e].c = kInvalidEntry;
        __syncthreads();

        /* phase B: replay the walk (bresenham.hpp:352-383 outer loop) up to the tile */
        if (threadIdx.x < n && my_count > 0) {
            const int s = threadIdx.x;
            const int my_base = base[s];
            const int ax = r.flags & kAxisY;
            const int sx = (r.flags & kStepXNeg) ? -1 : 1, sy = (r.flags & kStepYNeg) ? -1 : 1;
            const T t0 = r.t0, t1 = r.t1;
            const T d0t = sx > 0 ? t0 : -t0, d1t = sy > 0 ? t1 : -t1;   /* step * tau      */
            const T d0n = sx > 0 ? t1 : -t1, d1n = sy > 0 ? -t0 : t0;   /* step * normal   */
            const int far = sa > 0 ? c_hi : c_lo;
            int cx = r.x0, cy = r.y0;
            const int ex = r.x1, ey = r.y1;
            T te = r.te0, ne = r.ne0;
            long long guard = 0;
            while (cx != ex && cy != ey) {
                T exx = A::add(ne, d0n);
                T eyy = A::add(ne, d1n);
                T exy = A::add(exx, d1n);
                bool nx, ny;
                if (fabs(eyy) < fabs(exx)) { ny = true; nx = fabs(exy) < fabs(eyy); }
                else                       { nx = true; ny = fabs(exy) < fabs(exx); }
                if (ax ? ny : nx) {
                    const int c = ax ? cy : cx;
                    if (c >= c_lo && c <= c_hi) {
                        const int k = my_base + (c - c_begin) * sa;
                        Entry<T> en;
                        en.c = c;
                        en.sc = ax ? cx : cy;
                        en.te = te;
                        en.ne = ne;
                        ent[k] = en;
                        eslot[k] = (unsigned char)s;
                        if (c == far) break;
                    } else if ((c - far) * sa > 0) {
                        break;
                    }
                }
                if (nx) { cx += sx; te = A::add(te, d0t); ne = exx; }
                if (ny) { cy += sy; te = A::add(te, d1t); ne = A::add(ne, d1n); }
                if (++guard > 4LL * CBC_MAX_WALK + 64) {
                    atomicOr(&a.st->flags, 1 << CBC_ERR_RANGE);
                    break;
                }
            }
        }
        __syncthreads();

        /* phase C: the centre and both span halves of every entry (bresenham.hpp:364-381) */
        for (int e = threadIdx.x; e < total; e += kThreads) {
            const Entry<T> en = ent[e];
            if (en.c == kInvalidEntry) continue;
            const SlotParams<T> p = prm[eslot[e]];
            const int ax = p.axis;
            const int s_lo = ax ? x0 : y0, s_hi = ax ? x0 + tw - 1 : y0 + th - 1;
            T *trow = ax ? tile + ((ptrdiff_t)(en.c - y0) * tw - x0)
                         : tile + ((ptrdiff_t)(en.c - x0) - (ptrdiff_t)y0 * tw);
            const int sstride = ax ? 1 : tw;
            /* centre pixel: always visited */
            if (en.sc >= s_lo && en.sc <= s_hi) {
                T nf = A::normal_term(en.ne, p.len);
                T E = A::error(en.te, nf, p.len, p.len2, p.ww);
                if (E <= T(1)) {
                    T v = A::mul(a.max_val, A::template profile<K>(A::sqrt(E)));
                    T *dst = trow + (ptrdiff_t)en.sc * sstride;
                    if (OV == CBC_SUM) atomicAdd(dst, v); else combine_max(dst, v);
                }
            }
            #pragma unroll 1
            for (int half = 0; half < 2; half++) {
                const int h = half ? -p.ss : p.ss;
                if ((h > 0 && en.sc >= s_hi) || (h < 0 && en.sc <= s_lo)) continue;
                const T dt = h > 0 ? p.ts : -p.ts, dn = h > 0 ? p.ns : -p.ns;
                T te = en.te, ne = en.ne;
                int y = en.sc;
                for (int guard = 0; guard < 2 * CBC_MAX_WALK + 64; guard++) {
                    y += h;
                    te = A::add(te, dt);
                    ne = A::add(ne, dn);
                    T nf = A::normal_term(ne, p.len);
                    if (!(nf < p.ww)) break;
                    if (y >= s_lo && y <= s_hi) {
                        T E = A::error(te, nf, p.len, p.len2, p.ww);
                        if (E <= T(1)) {
                            T v = A::mul(a.max_val, A::template profile<K>(A::sqrt(E)));
                            T *dst = trow + (ptrdiff_t)y * sstride;
                            if (OV == CBC_SUM) atomicAdd(dst, v); else combine_max(dst, v);
                        }
                    }
                    if ((h > 0 && y >= s_hi) || (h < 0 && y <= s_lo)) break;
                }
            }
        }
        __syncthreads();
    }

    for (int e = threadIdx.x; e < tw * th; e += kThreads) {
        int r = e / tw, c = e - r * tw;
        gout[(size_t)r * g.W + c] = tile[e];
    }
}

/* ---- host side ----------------------------------------------------------------- */

thread_local std::string g_error;

/* opt-in per-stage event timing */
struct Profiler {
    std::mutex mu;
    bool enabled = false;
    std::vector<cudaEvent_t> pool;
    std::vector<std::vector<cudaEvent_t>> pending;   /* 5 events per call */
    double ms[4] = {0, 0, 0, 0};
    int calls = 0;

    cudaEvent_t get() {
        if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        return e;
    }
};

Profiler &profiler()
{
    static Profiler p;
    return p;
}

/* records event k (0..4) of the current call when profiling; no-op otherwise */
struct CallTimer {
    std::vector<cudaEvent_t> ev;
    cudaStream_t s;
    explicit CallTimer(cudaStream_t stream) : s(stream) {
        Profiler &p = profiler();
        std::lock_guard<std::mutex> g(p.mu);
        if (!p.enabled) return;
        for (int k = 0; k < 5; k++) ev.push_back(p.get());
    }
    void mark(int k) { if (!ev.empty() && ev[k]) cudaEventRecord(ev[k], s); }
    void commit() {
        if (ev.empty()) return;
        Profiler &p = profiler();
        std::lock_guard<std::mutex> g(p.mu);
        p.pending.push_back(ev);
        ev.clear();
    }
    ~CallTimer() {
        if (ev.empty()) return;
        Profiler &p = profiler();
        std::lock_guard<std::mutex> g(p.mu);
        for (cudaEvent_t e : ev) if (e) p.pool.push_back(e);
    }
};

int fail(int code, const std::string &msg)
{
    g_error = msg;
    return code;
}

struct Layout {
    size_t status, recs, counts, offsets, fillpos, pairs, total;
};

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct Resolved {
    int tile_w, tile_h, chunk, ent_cap;
};

bool resolve_tuning(const cbc_tuning *t, Resolved &r, std::string &why)
{
    r.tile_w = (t && t->tile_w) ? t->tile_w : kDefaultTileW;
    r.tile_h = (t && t->tile_h) ? t->tile_h : kDefaultTileH;
    r.chunk = (t && t->chunk_lines) ? t->chunk_lines : kDefaultChunk;
    if (r.tile_w < 16 || r.tile_w > 256 || (r.tile_w & 3)) { why = "tile_w must be a multiple of 4 in [16, 256]"; return false; }
    if (r.tile_h < 4 || r.tile_h > 256) { why = "tile_h must be in [4, 256]"; return false; }
    if (r.chunk < 1 || r.chunk > kMaxChunk) { why = "chunk_lines must be in [1, 32]"; return false; }
    r.ent_cap = r.chunk * (r.tile_w > r.tile_h ? r.tile_w : r.tile_h);
    return true;
}

Layout make_layout(long long n_frames, long long H, long long W, long long n_lines,
                   long long capacity, size_t rec_bytes, const Resolved &t)
{
    Layout L;
    long long tiles_x = (W + t.tile_w - 1) / t.tile_w, tiles_y = (H + t.tile_h - 1) / t.tile_h;
    long long n_bins = n_frames * tiles_x * tiles_y;
    size_t off = 0;
    L.status = off;  off = align_up(off + sizeof(DevStatus), 256);
    L.counts = off;  off = align_up(off + sizeof(int) * (size_t)n_bins, 256);
    L.offsets = off; off = align_up(off + sizeof(int) * (size_t)n_bins, 256);
    L.fillpos = off; off = align_up(off + sizeof(int) * (size_t)n_bins, 256);
    L.recs = off;    off = align_up(off + rec_bytes * (size_t)n_lines, 256);
    L.pairs = off;   off = align_up(off + sizeof(int) * (size_t)capacity, 256);
    L.total = off;
    return L;
}

template <typename T, int K, int OV>
cudaError_t launch_render(const RenderArgs<T> &ra, long long n_bins, size_t smem, cudaStream_t s)
{
    auto fn = render_kernel<T, K, OV>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    fn<<<(unsigned)n_bins, kThreads, smem, s>>>(ra);
    return cudaGetLastError();
}

template <typename T, int K>
cudaError_t launch_render_ov(const RenderArgs<T> &ra, int overlap, long long n_bins, size_t smem,
                             cudaStream_t s)
{
    return overlap == CBC_MAX ? launch_render<T, K, CBC_MAX>(ra, n_bins, smem, s)
                              : launch_render<T, K, CBC_SUM>(ra, n_bins, smem, s);
}

template <typename T>
cudaError_t launch_render_k(const RenderArgs<T> &ra, int kernel, int overlap, long long n_bins,
                            size_t smem, cudaStream_t s)
{
    switch (kernel) {
    case CBC_BIWEIGHT:    return launch_render_ov<T, CBC_BIWEIGHT>(ra, overlap, n_bins, smem, s);
    case CBC_GAUSSIAN:    return launch_render_ov<T, CBC_GAUSSIAN>(ra, overlap, n_bins, smem, s);
    case CBC_PARABOLIC:   return launch_render_ov<T, CBC_PARABOLIC>(ra, overlap, n_bins, smem, s);
    case CBC_RECTANGULAR: return launch_render_ov<T, CBC_RECTANGULAR>(ra, overlap, n_bins, smem, s);
    default:              return launch_render_ov<T, CBC_TRIANGULAR>(ra, overlap, n_bins, smem, s);
    }
}

template <typename T>
int draw_lines_impl(T *out, long long n_frames, long long H, long long W, const T *lines,
                    long long n_lines, const void *idxs, int idx_bytes, T max_val, int kernel,
                    int overlap, void *workspace, size_t ws_bytes, long long capacity,
                    const cbc_tuning *tuning, void *stream)
{
    g_error.clear();
    if (n_frames < 0 || H < 0 || W < 0 || n_lines < 0)
        return fail(CBC_ERR_INVALID, "negative size");
    if (H > INT_MAX / 2 || W > INT_MAX / 2)
        return fail(CBC_ERR_INVALID, "frame dimensions must be below 2^30");
    if (kernel < 0 || kernel > 4) return fail(CBC_ERR_INVALID, "Invalid kernel type");
    if (overlap != CBC_SUM && overlap != CBC_MAX)
        return fail(CBC_ERR_INVALID, "Invalid overlap keyword");
    if (idxs && idx_bytes != 4 && idx_bytes != 8)
        return fail(CBC_ERR_INVALID, "idx_bytes must be 4 or 8");
    if (!idxs && n_lines > 0 && n_frames != 1 && n_frames != n_lines)
        return fail(CBC_ERR_INVALID, "idxs has an incompatible size (" + std::to_string(n_lines) +
                                         " != " + std::to_string(n_frames) + ")");
    if (n_lines > 0 && (!out || !lines) && n_frames * H * W > 0)
        return fail(CBC_ERR_INVALID, "null pointer");
    if (capacity < 0 || capacity > INT_MAX) return fail(CBC_ERR_INVALID, "pair_capacity out of range");
    if (n_lines > INT_MAX) return fail(CBC_ERR_INVALID, "too many lines");
    Resolved t;
    std::string why;
    if (!resolve_tuning(tuning, t, why)) return fail(CBC_ERR_INVALID, why);
    Layout L = make_layout(n_frames, H, W, n_lines, capacity, sizeof(LineRec<T>), t);
    if (!workspace || ws_bytes < L.total)
        return fail(CBC_ERR_INVALID, "workspace too small (" + std::to_string(ws_bytes) + " < " +
                                         std::to_string(L.total) + ")");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    DevStatus *st = reinterpret_cast<DevStatus *>(ws + L.status);
    CallTimer timer(s);
    timer.mark(0);
    init_status_kernel<<<1, 1, 0, s>>>(st);
    cudaError_t e = cudaGetLastError();
    Geometry g;
    g.H = (int)H;
    g.W = (int)W;
    g.tile_w = t.tile_w;
    g.tile_h = t.tile_h;
    g.tiles_x = (int)((W + t.tile_w - 1) / t.tile_w);
    g.tiles_y = (int)((H + t.tile_h - 1) / t.tile_h);
    long long n_bins = n_frames * (long long)g.tiles_x * g.tiles_y;
    if (n_bins > INT_MAX) return fail(CBC_ERR_INVALID, "too many (frame, tile) bins");
    int *counts = reinterpret_cast<int *>(ws + L.counts);
    if (e == cudaSuccess && n_bins > 0) e = cudaMemsetAsync(counts, 0, sizeof(int) * n_bins, s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (n_lines == 0) return CBC_OK;
    LineRec<T> *recs = reinterpret_cast<LineRec<T> *>(ws + L.recs);
    unsigned nb_lines = (unsigned)((n_lines + kThreads - 1) / kThreads);
    if (!idxs || idx_bytes == 4)
        prep_kernel<T, int32_t><<<nb_lines, kThreads, 0, s>>>(lines, idxs, n_lines, n_frames, g,
                                                              recs, counts, st);
    else
        prep_kernel<T, int64_t><<<nb_lines, kThreads, 0, s>>>(lines, idxs, n_lines, n_frames, g,
                                                              recs, counts, st);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (n_bins == 0) return CBC_OK;
    timer.mark(1);
    int *offsets = reinterpret_cast<int *>(ws + L.offsets);
    int *fillpos = reinterpret_cast<int *>(ws + L.fillpos);
    int *pairs = reinterpret_cast<int *>(ws + L.pairs);
    offsets_kernel<<<(unsigned)((n_bins + kThreads - 1) / kThreads), kThreads, 0, s>>>(
        counts, offsets, fillpos, n_bins, capacity, st);
    timer.mark(2);
    fill_kernel<T><<<nb_lines, kThreads, 0, s>>>(recs, n_lines, g, fillpos, pairs, capacity, st);
    timer.mark(3);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    RenderArgs<T> ra;
    ra.out = out;
    ra.recs = recs;
    ra.counts = counts;
    ra.offsets = offsets;
    ra.pairs = pairs;
    ra.st = st;
    ra.g = g;
    ra.max_val = max_val;
    ra.chunk = t.chunk;
    ra.ent_cap = t.ent_cap;
    size_t smem = render_smem_bytes<T>(t.tile_w, t.tile_h, t.ent_cap);
    e = launch_render_k<T>(ra, kernel, overlap, n_bins, smem, s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    timer.mark(4);
    timer.commit();
    return CBC_OK;
}

}  // namespace cbc

extern "C" {

size_t cbc_draw_lines_workspace_size(int64_t n_frames, int64_t height, int64_t width,
                                     int64_t n_lines, int64_t pair_capacity, int32_t elem_bytes,
                                     const cbc_tuning *tuning)
{
    cbc::Resolved t;
    std::string why;
    if (!cbc::resolve_tuning(tuning, t, why)) return 0;
    if (n_frames < 0 || height < 0 || width < 0 || n_lines < 0 || pair_capacity < 0) return 0;
    size_t rec = elem_bytes == 8 ? sizeof(cbc::LineRec<double>) : sizeof(cbc::LineRec<float>);
    return cbc::make_layout(n_frames, height, width, n_lines, pair_capacity, rec, t).total;
}

int cbc_draw_lines_f32(float *out, int64_t n_frames, int64_t height, int64_t width,
                       const float *lines, int64_t n_lines, const void *idxs, int32_t idx_bytes,
                       float max_val, int32_t kernel, int32_t overlap, void *workspace,
                       size_t workspace_bytes, int64_t pair_capacity, const cbc_tuning *tuning,
                       void *stream)
{
    return cbc::draw_lines_impl<float>(out, n_frames, height, width, lines, n_lines, idxs,
                                       idx_bytes, max_val, kernel, overlap, workspace,
                                       workspace_bytes, pair_capacity, tuning, stream);
}

int cbc_draw_lines_f64(double *out, int64_t n_frames, int64_t height, int64_t width,
                       const double *lines, int64_t n_lines, const void *idxs, int32_t idx_bytes,
                       double max_val, int32_t kernel, int32_t overlap, void *workspace,
                       size_t workspace_bytes, int64_t pair_capacity, const cbc_tuning *tuning,
                       void *stream)
{
    return cbc::draw_lines_impl<double>(out, n_frames, height, width, lines, n_lines, idxs,
                                        idx_bytes, max_val, kernel, overlap, workspace,
                                        workspace_bytes, pair_capacity, tuning, stream);
}

int cbc_read_status(const void *workspace, cbc_status *status, void *stream)
{
    cbc::g_error.clear();
    if (!workspace || !status) return cbc::fail(CBC_ERR_INVALID, "null pointer");
    cbc::DevStatus d;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(&d, workspace, sizeof d, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cbc::fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    status->flags = d.flags;
    status->reserved = 0;
    status->bad_line = (int64_t)d.bad_line;
    status->idx_min = d.idx_min;
    status->idx_max = d.idx_max;
    status->pairs_needed = (int64_t)d.pairs;
    return CBC_OK;
}

int cbc_profile_enable(int32_t on)
{
    cbc::Profiler &p = cbc::profiler();
    std::lock_guard<std::mutex> g(p.mu);
    int prev = p.enabled ? 1 : 0;
    p.enabled = on != 0;
    return prev;
}

int cbc_profile_read(cbc_profile *profile, int32_t reset)
{
    cbc::g_error.clear();
    cbc::Profiler &p = cbc::profiler();
    std::lock_guard<std::mutex> g(p.mu);
    for (auto &ev : p.pending) {
        cudaError_t e = cudaEventSynchronize(ev[4]);
        if (e != cudaSuccess) return cbc::fail(CBC_ERR_CUDA, cudaGetErrorString(e));
        for (int k = 0; k < 4; k++) {
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, ev[k], ev[k + 1]) == cudaSuccess) p.ms[k] += ms;
        }
        p.calls++;
        for (cudaEvent_t x : ev) p.pool.push_back(x);
    }
    p.pending.clear();
    if (profile) {
        profile->calls = p.calls;
        profile->reserved = 0;
        profile->ms_prep = p.ms[0];
        profile->ms_offsets = p.ms[1];
        profile->ms_fill = p.ms[2];
        profile->ms_render = p.ms[3];
    }
    if (reset) {
        p.calls = 0;
        for (double &m : p.ms) m = 0.0;
    }
    return CBC_OK;
}

const char *cbc_last_error(void) { return cbc::g_error.c_str(); }

const char *cbc_version(void) { return CBC_VERSION; }

}  // extern "C"
