/*
 * cbc_lines3d.cu — draw_lines and accumulate_lines for 3-D lines (L = 7:
 * [x0, y0, z0, x1, y1, z1, width]) into volumes (F, D, H, W).
 *
 * Reference: the N = 3 instantiation of draw_lines_nd_impl / accumulate_lines_nd_impl
 * (cbclib_v2/_src/src/bresenham.cpp:38-101, :151-259) and its walk draw_line_3d
 * (bresenham.hpp:389-430) with LineIterator (:117-231) and BresenhamPlotter (:233-296).
 *
 * The 3-D walk visits, at every step of the long axis, the centre voxel and then four
 * quadrants: a 2-D walk over the two short axes that stays while the normal error is
 * below width^2, and from each of its voxels a 1-D span along each short axis.  Some
 * voxels are visited more than once, and with sum overlap each visit adds, as in the
 * reference.  Here the walk is replayed in the reference's arithmetic: float increments
 * as round-to-nearest intrinsics, and the error terms the reference rounds through
 * double (std::pow(T, int) promotes) reproduced bit for bit from float pairs, with a
 * double fallback near rounding ties (exact.cuh); the float64 overload computes them
 * in double.  The iterator's per-axis arrays are read and written through constant
 * indices only (at3 / put3 / increment_at for the line's run-time axes), which keeps
 * them in registers.
 *
 * Work split: prep3_kernel builds each line's record and walks its long axis once,
 * storing the exact iterator state at every long-axis column inside the volume;
 * render3_kernel then gives every (column, quadrant) to one thread, which draws it from
 * the column's checkpoint and combines each drawn voxel into `out` (sum: L2 add; max:
 * std::max merge; accumulate_lines with equal overlaps as in the 2-D path).
 * accumulate_lines with mixed overlaps builds each term in shared memory
 * (term_render3_kernel below).  The adjoint (cbc_draw_lines_3d_backward_*) replays the
 * same (column, quadrant) items with emitters that add each drawn voxel's gradient
 * term to its line (winner pass first for max overlap; adjoint3_kernel below).
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <limits.h>
#include <string>
#include <type_traits>

#include "cbc_accumulate.cuh"

namespace cbc {
namespace l3 {

/* pairs of axes: (0, 1), (0, 2), (1, 2) (UniquePairs<3>, geometry.hpp:403-448) */
__host__ __device__ constexpr int pair_a(int k) { return k == 2 ? 1 : 0; }
__host__ __device__ constexpr int pair_b(int k) { return k == 0 ? 1 : 2; }

/* a[i] and a[i] = v for a run-time axis i in [0, 3), written as selects over the three
 * constant indices: an array indexed only by constants stays in registers, one
 * indexed at run time is placed in local memory */
template <typename V>
__device__ __forceinline__ V at3(const V (&a)[3], int i)
{
    return i == 0 ? a[0] : (i == 1 ? a[1] : a[2]);
}

template <typename V>
__device__ __forceinline__ void put3(V (&a)[3], int i, V v)
{
    #pragma unroll
    for (int j = 0; j < 3; j++)
        if (j == i) a[j] = v;
}

template <typename T>
struct Rec3 {
    T tau[3];            /* pt1 - pt0                                   */
    T nrm[3][3];         /* normal of pair k, non-zero on its two axes  */
    T len, len2, w, ww;
    T rlen, rww;         /* RN(1 / len), RN(1 / ww) for the division shortcut */
    int32_t mpt1[3];     /* walk end (the reference adds one step)      */
    int32_t step[3];
    int32_t axis, frame, flags;
    int32_t c0, ncols, ck_base;
};

/* LineIterator state; `next` is recomputed from it by update() */
template <typename T>
struct It3 {
    int32_t cur[3];
    int32_t step[3];
    bool next[3];
    T te;
    T ne[3];
};

template <typename T>
struct Ck3 {
    int32_t cur[3];
    int32_t line;
    T te;
    T ne[3];
    int32_t seg;
    int32_t pad;
};

/* LineIterator::update with NormalError::is_next (bresenham.hpp:98-111, :205-220) */
template <typename T>
__device__ __forceinline__ void update(const Rec3<T> &r, It3<T> &it)
{
    using A = Ar<T>;
    #pragma unroll
    for (int i = 0; i < 3; i++) it.next[i] = it.step[i] != 0;
    #pragma unroll
    for (int k = 0; k < 3; k++) {
        const int a1 = pair_a(k), a2 = pair_b(k);
        if (it.step[a1] && it.step[a2]) {
            const T d1 = it.step[a1] > 0 ? r.nrm[k][a1] : -r.nrm[k][a1];
            const T d2 = it.step[a2] > 0 ? r.nrm[k][a2] : -r.nrm[k][a2];
            const T ex = A::add(it.ne[k], d1);
            const T ey = A::add(it.ne[k], d2);
            const T exy = A::add(ex, d2);
            bool f, s;
            if (fabs(ey) < fabs(ex)) { f = fabs(exy) < fabs(ey); s = true; }
            else                     { f = true; s = fabs(exy) < fabs(ex); }
            it.next[a1] = it.next[a1] && f;
            it.next[a2] = it.next[a2] && s;
        }
    }
}

/* LineIterator::increment by one step along `axis` (bresenham.hpp:195-203) */
template <typename T>
__device__ __forceinline__ void increment(const Rec3<T> &r, It3<T> &it, int axis)
{
    using A = Ar<T>;
    const int x = it.step[axis];
    it.cur[axis] += x;
    it.te = A::add(it.te, x > 0 ? r.tau[axis] : -r.tau[axis]);
    #pragma unroll
    for (int k = 0; k < 3; k++)
        if (pair_a(k) == axis || pair_b(k) == axis)
            it.ne[k] = A::add(it.ne[k], x > 0 ? r.nrm[k][axis] : -r.nrm[k][axis]);
}

/* increment() along a run-time axis: the constant-axis step under a predicate */
template <typename T>
__device__ __forceinline__ void increment_at(const Rec3<T> &r, It3<T> &it, int axis)
{
    #pragma unroll
    for (int j = 0; j < 3; j++)
        if (j == axis) increment(r, it, j);
}

template <typename T>
__device__ __forceinline__ void advance(const Rec3<T> &r, It3<T> &it)    /* operator++ */
{
    #pragma unroll
    for (int i = 0; i < 3; i++)
        if (it.next[i]) increment(r, it, i);
    update(r, it);
}

template <typename T>
__device__ __forceinline__ bool at_end(const Rec3<T> &r, const It3<T> &it)
{
    return it.cur[0] == r.mpt1[0] || it.cur[1] == r.mpt1[1] || it.cur[2] == r.mpt1[2];
}

/* BresenhamPlotter::normal_error (bresenham.hpp:284-289): a T accumulator fed with the
 * double squares of ne / len.  For float the double steps are reproduced from float
 * pairs (cbc_normal_error3*, exact.cuh), double arithmetic being a small fraction of
 * the float rate on this part. */
template <typename T>
__device__ __forceinline__ T normal_error(const Rec3<T> &r, const It3<T> &it)
{
    if constexpr (sizeof(T) == sizeof(float)) {
        return (r.flags & kFastDiv)
                   ? cbc_normal_error3_r(it.ne[0], it.ne[1], it.ne[2], r.len, r.rlen)
                   : cbc_normal_error3(it.ne[0], it.ne[1], it.ne[2], r.len);
    } else {
        const int fast = (r.flags & kFastDiv) ? 1 : 0;
        T err = T(0);
        #pragma unroll
        for (int k = 0; k < 3; k++) {
            const double b = Ar<double>::qdiv(it.ne[k], r.len, r.rlen, fast);
            err = (T)__dadd_rn((double)err, __dmul_rn(b, b));
        }
        return err;
    }
}

/* BresenhamPlotter::error (bresenham.hpp:291-296) from the position's normal error nf */
template <typename T>
__device__ __forceinline__ T error(const Rec3<T> &r, const It3<T> &it, T nf)
{
    if constexpr (sizeof(T) == sizeof(float)) {
        return (r.flags & kFastDiv)
                   ? cbc_pixel_error_r(it.te, nf, r.len, r.len2, r.ww, r.rlen, r.rww)
                   : cbc_pixel_error(it.te, nf, r.len, r.len2, r.ww);
    } else {
        using A = Ar<T>;
        const int fast = (r.flags & kFastDiv) ? 1 : 0;
        const T m1 = -it.te, m2 = A::sub(it.te, r.len2);
        T ta = m1 < m2 ? m2 : m1;
        ta = ta < T(0) ? T(0) : ta;
        const double a = Ar<double>::qdiv(ta, r.len, r.rlen, fast);
        const double e = __dadd_rn(__dmul_rn(a, a), (double)nf);
        return (T)Ar<double>::qdiv(e, r.ww, r.rww, fast);
    }
}

/* BresenhamPlotter construction and begin() (bresenham.hpp:243-263) */
template <typename T>
__device__ bool build_rec3(const T *ln, Rec3<T> &r, It3<T> &it, bool &too_long)
{
    using A = Ar<T>;
    too_long = false;
    T p0[3], p1[3];
    for (int i = 0; i < 3; i++) { p0[i] = ln[i]; p1[i] = ln[3 + i]; }
    const T w = ln[6];
    for (int i = 0; i < 7; i++)
        if (!isfinite(ln[i])) return false;
    if (!(w > T(0))) return false;                 /* error() is +inf everywhere */
    for (int i = 0; i < 3; i++) r.tau[i] = A::sub(p1[i], p0[i]);
    int ax = 0;
    for (int i = 1; i < 3; i++)
        if (fabs(at3(r.tau, ax)) < fabs(r.tau[i])) ax = i;
    r.axis = ax;
    T mag = T(0);
    for (int i = 0; i < 3; i++) mag = A::add(mag, A::mul(r.tau[i], r.tau[i]));
    r.len = A::sqrt(mag);
    if (!(r.len > T(0))) return false;
    const T ceilw = A::add(ceil(w), T(1));
    if (!(ceilw < T(1e9))) return false;
    T tn[3];
    for (int i = 0; i < 3; i++) tn[i] = A::div(r.tau[i], r.len);
    const T scale = fabs(A::div(ceilw, at3(tn, ax)));
    int32_t mpt0[3];
    const T lim = T(1 << 30);
    for (int i = 0; i < 3; i++) {
        r.step[i] = (p1[i] >= p0[i]) ? 1 : -1;
        const T a = round(A::sub(p0[i], A::mul(scale, tn[i])));
        const T b = round(A::add(p1[i], A::mul(scale, tn[i])));
        if (!(fabs(a) < lim && fabs(b) < lim)) { too_long = true; return false; }
        mpt0[i] = (int32_t)a;
        r.mpt1[i] = (int32_t)b + r.step[i];
    }
    long long walk = (long long)at3(r.mpt1, ax) - at3(mpt0, ax);
    if (walk < 0) walk = -walk;
    const T span = A::div(A::mul(w, r.len), fabs(at3(r.tau, ax)));
    if (walk > CBC_MAX_WALK || !(span < T(CBC_MAX_WALK))) { too_long = true; return false; }
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < 3; i++) r.nrm[k][i] = T(0);
    for (int k = 0; k < 3; k++) {
        const int a1 = pair_a(k), a2 = pair_b(k);
        r.nrm[k][a1] = A::sub(p1[a2], p0[a2]);
        r.nrm[k][a2] = A::sub(p0[a1], p1[a1]);
    }
    r.len2 = A::mul(r.len, r.len);
    r.w = w;
    r.ww = A::mul(w, w);
    T d[3];
    for (int i = 0; i < 3; i++) d[i] = A::sub((T)mpt0[i], p0[i]);
    it.te = T(0);
    for (int i = 0; i < 3; i++) it.te = A::add(it.te, A::mul(r.tau[i], d[i]));
    for (int k = 0; k < 3; k++) {
        T e = T(0);
        for (int i = 0; i < 3; i++) e = A::add(e, A::mul(r.nrm[k][i], d[i]));
        it.ne[k] = e;
    }
    for (int i = 0; i < 3; i++) { it.cur[i] = mpt0[i]; it.step[i] = r.step[i]; }
    update(r, it);
    r.rlen = A::rcp(r.len);
    r.rww = A::rcp(r.ww);
    r.flags = kDrawable | ((A::fast_range(r.len) && A::fast_range(r.ww)) ? kFastDiv : 0);
    return true;
}

struct Vol {
    int D, H, W;
    __device__ int ext(int axis) const { return axis == 0 ? W : (axis == 1 ? H : D); }
};

template <typename IdxT>
__device__ __forceinline__ long long load_frame(const void *idxs, long long i, long long n_frames)
{
    if (!idxs) return n_frames == 1 ? 0 : i;
    return (long long)static_cast<const IdxT *>(idxs)[i];
}

/* line records, frame checks and the long-axis checkpoints of every line */
template <typename T, typename IdxT>
__global__ void __launch_bounds__(kThreads)
prep3_kernel(const T *__restrict__ lines, const void *__restrict__ idxs, long long n_lines,
             long long n_frames, Vol v, Rec3<T> *__restrict__ recs, Ck3<T> *__restrict__ cks,
             long long ck_capacity, DevStatus *st)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = i < n_lines;
    long long frame = in ? load_frame<IdxT>(idxs, i, n_frames) : 0;
    if (idxs) warp_minmax(frame, in, st);
    Rec3<T> r;
    It3<T> it;
    r.flags = 0;
    r.ncols = 0;
    int nck = 0, lmin = 0, lmax = -1, sa = 1;
    if (in) {
        if (frame < 0 || frame >= n_frames) {
            atomicOr(&st->flags, 1 << CBC_ERR_INDEX);
            atomicMin(&st->bad_line, (unsigned long long)i);
        } else {
            bool too_long = false;
            if (build_rec3(lines + 7 * i, r, it, too_long)) {
                r.frame = (int32_t)frame;
                const int ax = r.axis;
                sa = at3(r.step, ax);
                const int first = at3(it.cur, ax), last = at3(r.mpt1, ax) - sa;
                lmin = max(min(first, last), 0);
                lmax = min(max(first, last), v.ext(ax) - 1);
                if (lmin <= lmax) {
                    r.ncols = lmax - lmin + 1;
                    r.c0 = sa > 0 ? lmin : lmax;
                    nck = r.ncols;
                } else {
                    r.flags = 0;
                }
            } else if (too_long) {
                atomicOr(&st->flags, 1 << CBC_ERR_RANGE);
                atomicMin(&st->bad_line, (unsigned long long)i);
            }
        }
    }
    const int lane = threadIdx.x & 31;
    int incl = nck;
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    unsigned long long wbase = 0;
    if (lane == 31) wbase = atomicAdd(&st->cks, (unsigned long long)incl);
    wbase = __shfl_sync(0xffffffffu, wbase, 31);
    if (!in) return;
    if (nck > 0) {
        const unsigned long long cb = wbase + (unsigned long long)(incl - nck);
        if (cb + (unsigned long long)nck > (unsigned long long)ck_capacity) {
            atomicOr(&st->flags, 1 << CBC_ERR_CAPACITY);
            nck = 0;
            r.flags = 0;
        } else {
            r.ck_base = (int32_t)cb;
        }
    }
    if (nck > 0) {
        /* columns are the positions where the next step moves the long axis; one per
         * long coordinate.  Checkpoint k holds the state at the column of walk index k
         * (walk index = (c - c0) * step of the long axis), so the renders start every
         * column or quadrant from its own checkpoint without walking. */
        const int ax = r.axis;
        int k = 0;
        long long guard = 0;
        while (k < nck && !at_end(r, it)) {
            if (at3(it.next, ax)) {
                const int idx = (at3(it.cur, ax) - r.c0) * sa;
                if (idx == k) {
                    Ck3<T> c;
                    for (int a = 0; a < 3; a++) c.cur[a] = it.cur[a];
                    c.line = (int32_t)i;
                    c.te = it.te;
                    for (int a = 0; a < 3; a++) c.ne[a] = it.ne[a];
                    c.seg = k;
                    c.pad = 0;
                    cks[r.ck_base + k] = c;
                    k++;
                }
            }
            advance(r, it);
            if (++guard > 4LL * CBC_MAX_WALK + 64) {
                atomicOr(&st->flags, 1 << CBC_ERR_RANGE);
                break;
            }
        }
        for (; k < nck; k++) {          /* the walk ended first: empty segments */
            Ck3<T> c;
            c.cur[0] = INT_MIN;
            c.cur[1] = c.cur[2] = 0;
            c.line = (int32_t)i;
            c.te = T(0);
            c.ne[0] = c.ne[1] = c.ne[2] = T(0);
            c.seg = k;
            c.pad = 0;
            cks[r.ck_base + k] = c;
        }
    }
    recs[i] = r;
}

/* where the drawn voxels go */
template <typename T, int K>
struct Emit3 {
    T *out;
    T max_val;
    int mode;                      /* 0 sum, 1 max (draw_lines); accumulate: kAcc* + 4 */
    const int *term_of_line;
    unsigned long long *keys;
    T *vals;
    unsigned long long mask;
    const int *tbig;               /* mixed overlaps: the terms this pass draws */
    DevStatus *st;
    __device__ __forceinline__ bool table_mode() const {
        return mode == 4 + kAccMaxSum || mode == 4 + kAccSumMax;
    }
    __device__ __forceinline__ void operator()(long long fbase, long long vox, int line, T E) const {
        using A = Ar<T>;
        const T v = A::mul(max_val, A::template profile<K>(A::sqrt(E)));
        switch (mode) {
        case 0:  atomicAdd(out + fbase + vox, v); break;
        case 1:  global_combine_max(out + fbase + vox, v); break;
        case 4 + kAccSumSum: atomicAdd(out + fbase + vox, v); break;
        case 4 + kAccMaxSum:
            table_combine<T, 1>(keys, vals, mask, term_of_line[line], vox, v, st);
            break;
        case 4 + kAccSumMax:
            table_combine<T, 0>(keys, vals, mask, term_of_line[line], vox, v, st);
            break;
        default:  global_combine_max(out + fbase + vox, T(0) < v ? v : T(0)); break;
        }
    }
};

/* emitters that need the voxel's coordinates (the adjoint) define voxel(...) */
template <class EM, class = void> struct TakesCoords : std::false_type {};
template <class EM>
struct TakesCoords<EM, std::void_t<decltype(&EM::voxel)>> : std::true_type {};

/* a visited voxel with normal error nf: inside the volume and with error <= 1, the emit */
template <typename T, class EM>
__device__ __forceinline__ void visit(const Rec3<T> &r, const It3<T> &it, T nf, const Vol &v,
                                      long long fbase, int line, const EM &emit)
{
    if (it.cur[0] < 0 || it.cur[0] >= v.W || it.cur[1] < 0 || it.cur[1] >= v.H ||
        it.cur[2] < 0 || it.cur[2] >= v.D)
        return;
    const T E = error(r, it, nf);
    if (!(E <= T(1))) return;
    const long long vox = ((long long)it.cur[2] * v.H + it.cur[1]) * v.W + it.cur[0];
    if constexpr (TakesCoords<EM>::value) emit.voxel(fbase, vox, line, E, it.cur);
    else emit(fbase, vox, line, E);
}

template <typename T>
__device__ __forceinline__ It3<T> collapse(const Rec3<T> &r, const It3<T> &src, int axis)
{
    It3<T> it = src;
    put3(it.step, axis, 0);
    update(r, it);
    return it;
}

/* the start of quadrant q's 2-D walk over the short-axis plane (bresenham.hpp:409-412):
 * the column's iterator without its long axis, flipped on the quadrant's axes, moved
 * one step */
template <typename T>
__device__ __forceinline__ It3<T> quadrant_start(const Rec3<T> &r, const It3<T> &it, int q)
{
    const int ax = r.axis, ax1 = (ax + 1) % 3, ax2 = (ax + 2) % 3;
    It3<T> ixy = it;
    put3(ixy.step, ax, 0);
    if (q & 1) put3(ixy.step, ax1, -at3(ixy.step, ax1));
    if (q >> 1) put3(ixy.step, ax2, -at3(ixy.step, ax2));
    update(r, ixy);
    increment_at(r, ixy, ((q & 1) ^ (q >> 1)) == 0 ? ax1 : ax2);      /* move */
    update(r, ixy);
    return ixy;
}

/* quadrants [q0, q1) of a column of draw_line_3d (bresenham.hpp:392-428), with the
 * centre voxel when q0 is 0.  The reference's nested loops (the quadrant's 2-D walk
 * while normal_error < width^2, from each of its positions a 1-D span along each
 * short axis with a next step) are run as one loop that looks at one position per
 * iteration: the centre, a 2-D walk position (mode 0) or a span position (mode 1).
 * Each iteration evaluates one normal error and makes at most one visit, so the lanes
 * of a warp, wherever they are in their walks, share the expensive part of the
 * iteration; the visit order is the reference's. */
template <typename T, class EM>
__device__ __forceinline__ void draw_quadrants(const Rec3<T> &r, const It3<T> &it, int q0,
                                               int q1, const Vol &v, long long fbase, int line,
                                               const EM &emit, DevStatus *st)
{
    const int ax = r.axis;
    int q = q0, mode = 0, j = 0;
    bool centre = q0 == 0;
    It3<T> ixy = quadrant_start(r, it, q);
    It3<T> ix = ixy;
    long long guard = 0;
    for (;;) {
        const It3<T> cur = centre ? it : (mode ? ix : ixy);
        const T nf = normal_error(r, cur);
        const bool in = centre || nf < r.ww;
        if (in) visit(r, cur, nf, v, fbase, line, emit);
        /* the transition: which iterator steps next (one advance site for both) */
        bool step = true;
        if (centre) {
            centre = false;                      /* then quadrant q0's first position */
            step = false;
        } else if (mode == 0 || !in) {
            if (mode == 0 && !in) {              /* the quadrant's 2-D walk has ended */
                if (++q >= q1) return;
                ixy = quadrant_start(r, it, q);
                step = false;
            } else {
                j = mode == 0 ? 1 : j + 1;       /* a new position, or a span ended */
                /* the next span from the current 2-D position, else its next position */
                mode = 0;
                for (; j < 3; j++) {
                    const int aj = (ax + j) % 3;
                    if (at3(ixy.next, aj)) {
                        ix = collapse(r, ixy, aj);
                        mode = 1;
                        break;
                    }
                }
            }
        }
        if (step) {
            It3<T> nxt = mode ? ix : ixy;
            advance(r, nxt);
            if (mode) ix = nxt;
            else ixy = nxt;
        }
        if (++guard > 8LL * CBC_MAX_WALK) {
            atomicOr(&st->flags, 1 << CBC_ERR_RANGE);
            return;
        }
    }
}

/* the iterator at a column from the column's checkpoint */
template <typename T>
__device__ __forceinline__ It3<T> column_iter(const Rec3<T> &r, const Ck3<T> &ck)
{
    It3<T> it;
    #pragma unroll
    for (int i = 0; i < 3; i++) { it.cur[i] = ck.cur[i]; it.step[i] = r.step[i]; }
    it.te = ck.te;
    #pragma unroll
    for (int i = 0; i < 3; i++) it.ne[i] = ck.ne[i];
    update(r, it);
    return it;
}

template <typename T>
struct Render3Args {
    const Rec3<T> *recs;
    const Ck3<T> *cks;
    Vol v;
    DevStatus *st;
    const int *nbig;               /* mixed overlaps: terms through the workspace table */
    const float *big_est;          /* and their estimated pairs                        */
    long long table_capacity;
};

/* one thread per (column, quadrant), quadrant-major (the lanes of a warp take the same
 * quadrant of consecutive columns; adjacent lanes on one column's four quadrants would
 * collide on the voxels the quadrants share), grid-stride; quadrant 0 also takes the
 * centre voxel */
template <typename T, int K>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 3 : 2)
render3_kernel(Render3Args<T> a, Emit3<T, K> emit)
{
    if (a.st->flags & kFatal) return;
    const bool table = emit.table_mode();
    if (table && !table_terms_fit(a.nbig, a.big_est, a.table_capacity, a.st)) return;
    const long long ncks = (long long)a.st->cks, total = 4 * ncks;
    for (long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x; item < total;
         item += (long long)gridDim.x * blockDim.x) {
        const int q = (int)(item / ncks);
        const Ck3<T> ck = a.cks[item - (long long)q * ncks];
        if (ck.cur[0] == INT_MIN) continue;
        if (table && !emit.tbig[emit.term_of_line[ck.line]]) continue;
        const Rec3<T> r = a.recs[ck.line];
        const It3<T> it = column_iter(r, ck);
        const long long fbase = (long long)r.frame * a.v.D * a.v.H * a.v.W;
        draw_quadrants(r, it, q, q + 1, a.v, fbase, ck.line, emit, a.st);
    }
}

/* ---- accumulate with mixed overlaps: terms combined in shared memory ----
 * A term's lines are combined with in_overlap in a zeroed buffer before the buffer is
 * merged into its frame (bresenham.cpp:151-259).  Here one CTA takes one term at a
 * time and builds that buffer as an open-addressing (voxel, value) table in shared
 * memory: the term's columns (and quadrants of columns) are shared out among the
 * threads, each starting from the column's own checkpoint, every visited voxel is combined into its slot (in-term max or sum), and afterwards each
 * drawn voxel is merged into the volume with one global atomic.  A term with more
 * voxels than the table takes is done in partitions of its voxels (a hash of the voxel
 * index modulo P; each pass walks all of the term's columns and keeps the voxels of
 * one partition): P starts from an estimate, and a partition that fills the table is
 * split in two and redone, so every voxel is merged exactly once.  Terms whose estimate
 * needs more than kTermMaxParts partitions go instead through the workspace (term,
 * voxel) table in render3_kernel, sized by the call (CBC_ERR_CAPACITY names the
 * capacity to retry with). */
template <typename T> struct TermTable { static constexpr int kBits = 13; };   /* 64 KB */
template <> struct TermTable<double> { static constexpr int kBits = 12; };       /* 48 KB */
constexpr int kTermThreads = 256;
constexpr int kTermChunk = kTermThreads;      /* lines staged per chunk */
constexpr int kTermStack = 64;                /* pending partitions per term */
constexpr int kTermMaxParts = 8;              /* larger terms use the workspace table */

template <typename T>
struct TermArgs {
    const Rec3<T> *recs;
    const Ck3<T> *cks;
    Vol v;
    DevStatus *st;
    T *out;
    T max_val;
    const int *tcount, *toff, *tlines, *tbig, *frame_of_term;
    const float *test;
    long long n_terms;
};

template <typename T>
constexpr size_t term_smem()
{
    return (size_t)(1 << TermTable<T>::kBits) * (sizeof(int) + sizeof(T));
}

/* after prep3: each drawable line adds itself to its term's count and a typical voxel
 * count, columns x pi (0.9 w + 0.5)^2, to the term's estimate (only the starting
 * number of partitions depends on it) */
template <typename T>
__global__ void __launch_bounds__(kThreads)
term_count3_kernel(const Rec3<T> *__restrict__ recs, const int *__restrict__ term_of_line,
                   long long n_lines, int *__restrict__ tcount, float *__restrict__ test)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_lines || recs[i].ncols <= 0) return;
    const int t = term_of_line[i];
    atomicAdd(&tcount[t], 1);
    const float r = 0.9f * (float)recs[i].w + 0.5f;
    atomicAdd(&test[t], (float)recs[i].ncols * 3.14159265f * r * r);
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
term_fill3_kernel(const Rec3<T> *__restrict__ recs, const int *__restrict__ term_of_line,
                  long long n_lines, int *__restrict__ tfill, int *__restrict__ tlines)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_lines || recs[i].ncols <= 0) return;
    tlines[atomicAdd(&tfill[term_of_line[i]], 1)] = (int)i;
}

/* a term's voxels of the current partition into the shared table; `count` grows with
 * every claimed slot and `full` is raised at 3/4 of the table */
template <typename T, int K, int IN_MAX>
struct SmEmit {
    int *key;
    T *val;
    int *count;
    int *full;
    T max_val;
    unsigned pmask, part;
    __device__ __forceinline__ void operator()(long long, long long vox, int, T E) const {
        using A = Ar<T>;
        constexpr int kBits = TermTable<T>::kBits, kSize = 1 << kBits;
        const int k = (int)vox;
        if ((part_hash((unsigned)k) & pmask) != part) return;
        if (*reinterpret_cast<volatile int *>(full)) return;    /* this pass is redone */
        const T v = A::mul(max_val, A::template profile<K>(A::sqrt(E)));
        unsigned h = ((unsigned)k * 2654435761u) >> (32 - kBits);   /* Fibonacci hashing */
        for (int p = 0; p < kSize; p++) {
            int cur = *reinterpret_cast<volatile int *>(key + h);
            if (cur == -1) {
                cur = atomicCAS(key + h, -1, k);
                if (cur == -1 && atomicAdd(count, 1) >= kSize * 3 / 4)
                    *reinterpret_cast<volatile int *>(full) = 1;
            }
            if (cur == -1 || cur == k) {
                if (IN_MAX) term_combine_max(val + h, v);
                else atomicAdd(val + h, v);
                return;
            }
            h = (h + 1) & (kSize - 1);
        }
        *reinterpret_cast<volatile int *>(full) = 1;
    }
};

template <typename T, int K, int IN_MAX, int OUT_MAX>
__global__ void __launch_bounds__(kTermThreads, 3)
term_render3_kernel(TermArgs<T> a)
{
    constexpr int kSize = 1 << TermTable<T>::kBits;
    extern __shared__ __align__(16) unsigned char term_smem_raw[];
    T *s_val = reinterpret_cast<T *>(term_smem_raw);
    int *s_key = reinterpret_cast<int *>(term_smem_raw + sizeof(T) * kSize);
    __shared__ int s_pre[kTermChunk + 1];
    __shared__ int s_line[kTermChunk];
    __shared__ int s_warp[kTermThreads / 32];
    __shared__ unsigned s_stack[kTermStack];
    __shared__ int s_depth, s_count, s_full;
    if (a.st->flags & kFatal) return;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const long long frame_vox = (long long)a.v.D * a.v.H * a.v.W;
    for (long long t = blockIdx.x; t < a.n_terms; t += gridDim.x) {
        const int n_t = a.tcount[t];
        if (n_t == 0 || a.tbig[t]) continue;
        /* pending partitions (part, log2 P), one per 32-bit word */
        if (tid == 0) {
            /* at most kTermMaxParts starting partitions: with one more entry per split,
             * the stack stays below kTermMaxParts + 24 entries */
            const float want = a.test[t] / (0.6f * (float)kSize);
            int lg = 0;
            while ((float)(1 << lg) < want && (1 << lg) < kTermMaxParts) lg++;
            s_depth = 0;
            for (int p = (1 << lg) - 1; p >= 0; p--) s_stack[s_depth++] = ((unsigned)p << 5) | lg;
        }
        __syncthreads();
        while (s_depth > 0) {
            const unsigned top = s_stack[s_depth - 1];
            const unsigned lg = top & 31u, part = top >> 5;
            for (int j = tid; j < kSize; j += kTermThreads) {
                s_key[j] = -1;
                s_val[j] = T(0);
            }
            if (tid == 0) {
                s_count = 0;
                s_full = 0;
            }
            __syncthreads();
            const SmEmit<T, K, IN_MAX> emit{s_key, s_val, &s_count, &s_full, a.max_val,
                                            (1u << lg) - 1u, part};
            for (int c0 = 0; c0 < n_t && !s_full; c0 += kTermChunk) {
                /* this chunk's lines and the prefix sum of their columns */
                const int nc = min(kTermChunk, n_t - c0);
                int ncol = 0;
                if (tid < nc) {
                    const int l = a.tlines[a.toff[t] + c0 + tid];
                    s_line[tid] = l;
                    ncol = a.recs[l].ncols;
                }
                int incl = ncol;
                for (int o = 1; o < 32; o <<= 1) {
                    const int u = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += u;
                }
                if (lane == 31) s_warp[wid] = incl;
                __syncthreads();
                int before = 0;
                for (int w = 0; w < wid; w++) before += s_warp[w];
                s_pre[tid] = before + incl - ncol;
                if (tid == kTermThreads - 1) s_pre[kTermThreads] = before + incl;
                __syncthreads();
                const int total = s_pre[nc];
                /* items from the columns' own checkpoints: whole columns while every
                 * thread has one, then the columns of the last, partial round split into
                 * their four quadrants (quadrant-major), which shortens that round to
                 * about a quadrant's time */
                const int full = total / kTermThreads * kTermThreads, rest = total - full;
                const int items = full + 4 * rest;
                for (int j = tid; j < items && !*reinterpret_cast<volatile int *>(&s_full);
                     j += kTermThreads) {
                    int c = j, q0 = 0, q1 = 4;
                    if (j >= full) {
                        q0 = (j - full) / rest;
                        q1 = q0 + 1;
                        c = full + (j - full - q0 * rest);
                    }
                    int lo = 0, hi = nc - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (s_pre[mid] <= c) lo = mid;
                        else hi = mid - 1;
                    }
                    const int line = s_line[lo], col = c - s_pre[lo];
                    const Rec3<T> r = a.recs[line];
                    const Ck3<T> ck = a.cks[r.ck_base + col];
                    if (ck.cur[0] == INT_MIN) continue;
                    draw_quadrants(r, column_iter(r, ck), q0, q1, a.v, 0, line, emit, a.st);
                }
                __syncthreads();
            }
            if (s_full) {
                /* too many voxels in this partition: split it, nothing merged */
                if (tid == 0) {
                    s_depth--;
                    if (lg < 24 && s_depth + 2 <= kTermStack) {
                        s_stack[s_depth++] = ((part + (1u << lg)) << 5) | (lg + 1);
                        s_stack[s_depth++] = (part << 5) | (lg + 1);
                    } else {
                        atomicOr(&a.st->flags, 1 << CBC_ERR_CAPACITY);
                    }
                }
            } else {
                T *dst = a.out + (long long)a.frame_of_term[t] * frame_vox;
                for (int j = tid; j < kSize; j += kTermThreads) {
                    const int k = s_key[j];
                    if (k < 0) continue;
                    if (OUT_MAX) global_combine_max(dst + k, s_val[j]);
                    else atomicAdd(dst + k, s_val[j]);
                }
                if (tid == 0) s_depth--;
            }
            __syncthreads();
        }
    }
}

struct Layout3 {
    size_t status, recs, cks, frame_of_line, term_of_line, frame_of_term, keys, vals;
    size_t tcount, toff, tfill, test, tlines, tbig, counters, total;
};

inline Layout3 layout3(long long n_lines, long long n_terms, long long ck_capacity,
                       long long table_capacity, size_t elem)
{
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t rec = elem == 4 ? sizeof(Rec3<float>) : sizeof(Rec3<double>);
    const size_t ck = elem == 4 ? sizeof(Ck3<float>) : sizeof(Ck3<double>);
    Layout3 L;
    size_t off = 0;
    L.status = off;        off = up(off + sizeof(DevStatus));
    L.recs = off;          off = up(off + rec * (size_t)n_lines);
    L.cks = off;           off = up(off + ck * (size_t)ck_capacity);
    L.frame_of_line = off; off = up(off + sizeof(int) * (size_t)n_lines);
    L.term_of_line = off;  off = up(off + sizeof(int) * (size_t)n_lines);
    L.frame_of_term = off; off = up(off + sizeof(int) * (size_t)n_terms);
    L.keys = off;          off = up(off + sizeof(unsigned long long) * (size_t)table_capacity);
    L.vals = off;          off = up(off + elem * (size_t)table_capacity);
    L.tcount = off;        off = up(off + sizeof(int) * (size_t)n_terms);
    L.toff = off;          off = up(off + sizeof(int) * (size_t)n_terms);
    L.tfill = off;         off = up(off + sizeof(int) * (size_t)n_terms);
    L.test = off;          off = up(off + sizeof(float) * (size_t)n_terms);
    L.tlines = off;        off = up(off + sizeof(int) * (size_t)(n_terms > 0 ? n_lines : 0));
    L.tbig = off;          off = up(off + sizeof(int) * (size_t)n_terms);
    L.counters = off;      off = up(off + 16);    /* cursor, table terms, their pairs */
    L.total = off;
    return L;
}

template <typename T, int K>
cudaError_t launch_render3(const Render3Args<T> &a, const Emit3<T, K> &emit, cudaStream_t s)
{
    const unsigned grid = resident_grid(render3_kernel<T, K>, kThreads);
    render3_kernel<T, K><<<grid, kThreads, 0, s>>>(a, emit);
    note_launches(1);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_render3_k(const Render3Args<T> &a, int kernel, T *out, T max_val, int mode,
                             const int *term_of_line, unsigned long long *keys, T *vals,
                             unsigned long long mask, const int *tbig, cudaStream_t s)
{
#define CBC_L3_CASE(KK)                                                                  \
    case KK: {                                                                           \
        Emit3<T, KK> e{out, max_val, mode, term_of_line, keys, vals, mask, tbig, a.st};  \
        return launch_render3<T, KK>(a, e, s);                                           \
    }
    switch (kernel) {
    CBC_L3_CASE(CBC_BIWEIGHT)
    CBC_L3_CASE(CBC_GAUSSIAN)
    CBC_L3_CASE(CBC_PARABOLIC)
    CBC_L3_CASE(CBC_RECTANGULAR)
    default: {
        Emit3<T, CBC_TRIANGULAR> e{out, max_val, mode, term_of_line, keys, vals, mask, tbig,
                                    a.st};
        return launch_render3<T, CBC_TRIANGULAR>(a, e, s);
    }
    }
#undef CBC_L3_CASE
}

/* shared by draw and accumulate: frames given per line (int32 frame_of_line or the
 * caller's idxs), accumulate state when mode >= 4 */
template <typename T, int K, int IN_MAX, int OUT_MAX>
cudaError_t launch_terms3(const TermArgs<T> &ta, cudaStream_t s)
{
    auto fn = term_render3_kernel<T, K, IN_MAX, OUT_MAX>;
    constexpr size_t smem = term_smem<T>();
    static std::atomic<int> grid_cache[64];
    int dev = 0;
    cudaGetDevice(&dev);
    int g = grid_cache[dev & 63].load(std::memory_order_relaxed);
    if (g == 0) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kTermThreads, smem);
        g = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
        grid_cache[dev & 63].store(g, std::memory_order_relaxed);
    }
    const long long grid = ta.n_terms < g ? ta.n_terms : g;
    if (grid < 1) return cudaSuccess;
    fn<<<(unsigned)grid, kTermThreads, smem, s>>>(ta);
    note_launches(1);
    return cudaGetLastError();
}

template <typename T, int K>
cudaError_t launch_terms3_k(const TermArgs<T> &ta, int acc, cudaStream_t s)
{
    return acc == kAccMaxSum ? launch_terms3<T, K, 1, 0>(ta, s) : launch_terms3<T, K, 0, 1>(ta, s);
}

/* the mixed-overlap accumulate: line lists per term; the terms too large for shared
 * memory through the workspace table (render3_kernel's table modes, then the merge),
 * the others in shared memory */
template <typename T>
cudaError_t run_terms3(const Render3Args<T> &ra, T *out, T max_val, int kernel, int acc,
                       long long n_lines, long long n_terms, const int *term_of_line,
                       const int *frame_of_term, unsigned long long *keys, T *vals,
                       long long table_capacity, unsigned char *ws, const Layout3 &L,
                       cudaStream_t s)
{
    int *tcount = reinterpret_cast<int *>(ws + L.tcount);
    int *toff = reinterpret_cast<int *>(ws + L.toff);
    int *tfill = reinterpret_cast<int *>(ws + L.tfill);
    int *tlines = reinterpret_cast<int *>(ws + L.tlines);
    int *tbig = reinterpret_cast<int *>(ws + L.tbig);
    float *test = reinterpret_cast<float *>(ws + L.test);
    unsigned long long *cursor = reinterpret_cast<unsigned long long *>(ws + L.counters);
    int *nbig = reinterpret_cast<int *>(ws + L.counters + 8);
    float *big_est = reinterpret_cast<float *>(ws + L.counters + 12);
    cudaError_t e = cudaMemsetAsync(tcount, 0, sizeof(int) * (size_t)n_terms, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(test, 0, sizeof(float) * (size_t)n_terms, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ws + L.counters, 0, 16, s);
    if (e == cudaSuccess && table_capacity > 0) e = clear_table(keys, vals, table_capacity, s);
    if (e != cudaSuccess) return e;
    const unsigned nbl = (unsigned)((n_lines + kThreads - 1) / kThreads);
    const unsigned nbt = (unsigned)((n_terms + kThreads - 1) / kThreads);
    term_count3_kernel<T><<<nbl, kThreads, 0, s>>>(ra.recs, term_of_line, n_lines, tcount, test);
    term_offsets_kernel<<<nbt, kThreads, 0, s>>>(tcount, toff, tfill, n_terms, cursor);
    term_fill3_kernel<T><<<nbl, kThreads, 0, s>>>(ra.recs, term_of_line, n_lines, tfill, tlines);
    term_class_kernel<<<nbt, kThreads, 0, s>>>(
        tcount, test, n_terms, (float)kTermMaxParts * 0.6f * (float)(1 << TermTable<T>::kBits),
        tbig, nbig, big_est);
    note_launches(4);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    Render3Args<T> a = ra;
    a.nbig = nbig;
    a.big_est = big_est;
    a.table_capacity = table_capacity;
    const unsigned long long mask = table_capacity > 0 ? (unsigned long long)table_capacity - 1 : 0;
    e = launch_render3_k<T>(a, kernel, out, max_val, 4 + acc, term_of_line, keys, vals, mask,
                            tbig, s);
    if (e != cudaSuccess) return e;
    TermArgs<T> ta{ra.recs, ra.cks, ra.v, ra.st, out, max_val, tcount, toff, tlines, tbig,
                   frame_of_term, test, n_terms};
    switch (kernel) {
    case CBC_BIWEIGHT:    e = launch_terms3_k<T, CBC_BIWEIGHT>(ta, acc, s); break;
    case CBC_GAUSSIAN:    e = launch_terms3_k<T, CBC_GAUSSIAN>(ta, acc, s); break;
    case CBC_PARABOLIC:   e = launch_terms3_k<T, CBC_PARABOLIC>(ta, acc, s); break;
    case CBC_RECTANGULAR: e = launch_terms3_k<T, CBC_RECTANGULAR>(ta, acc, s); break;
    default:              e = launch_terms3_k<T, CBC_TRIANGULAR>(ta, acc, s); break;
    }
    if (e == cudaSuccess && table_capacity > 0)
        e = launch_merge(out, keys, vals, table_capacity, frame_of_term,
                         (long long)ra.v.D * ra.v.H * ra.v.W, acc == kAccSumMax, ra.st, s);
    return e;
}

template <typename T>
int run3(T *out, long long n_frames, long long D, long long H, long long W, const T *lines,
         long long n_lines, const void *idxs, int idx_bytes, T max_val, int kernel, int mode,
         unsigned char *ws, const Layout3 &L, long long ck_capacity, long long table_capacity,
         const int *term_of_line, const int *frame_of_term, cudaStream_t s,
         long long n_terms = 0)
{
    DevStatus *st = reinterpret_cast<DevStatus *>(ws + L.status);
    Rec3<T> *recs = reinterpret_cast<Rec3<T> *>(ws + L.recs);
    Ck3<T> *cks = reinterpret_cast<Ck3<T> *>(ws + L.cks);
    Vol v{(int)D, (int)H, (int)W};
    const unsigned nb = (unsigned)((n_lines + kThreads - 1) / kThreads);
    const bool terms = mode == 4 + kAccMaxSum || mode == 4 + kAccSumMax;
    if (idxs && idx_bytes == 8)
        prep3_kernel<T, int64_t><<<nb, kThreads, 0, s>>>(lines, idxs, n_lines, n_frames, v, recs,
                                                         cks, ck_capacity, st);
    else
        prep3_kernel<T, int32_t><<<nb, kThreads, 0, s>>>(lines, idxs, n_lines, n_frames, v, recs,
                                                         cks, ck_capacity, st);
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    Render3Args<T> a{recs, cks, v, st, nullptr, nullptr, 0};
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(ws + L.keys);
    T *vals = reinterpret_cast<T *>(ws + L.vals);
    if (terms) {
        if (n_terms > 0) {
            e = run_terms3<T>(a, out, max_val, kernel, mode - 4, n_lines, n_terms, term_of_line,
                              frame_of_term, keys, vals, table_capacity, ws, L, s);
            if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
        }
        return CBC_OK;
    }
    e = launch_render3_k<T>(a, kernel, out, max_val, mode, term_of_line, keys, vals, 0, nullptr, s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    return CBC_OK;
}

template <typename T>
int draw3_impl(T *out, long long n_frames, long long D, long long H, long long W, const T *lines,
               long long n_lines, const void *idxs, int idx_bytes, T max_val, int kernel,
               int overlap, void *workspace, size_t ws_bytes, long long ck_capacity, void *stream)
{
    clear_error();
    if (n_frames < 0 || D < 0 || H < 0 || W < 0 || n_lines < 0)
        return fail(CBC_ERR_INVALID, "negative size");
    if (kernel < CBC_BIWEIGHT || kernel > CBC_TRIANGULAR)
        return fail(CBC_ERR_INVALID, "kernel is missing");
    if (overlap != CBC_SUM && overlap != CBC_MAX) return fail(CBC_ERR_INVALID, "Invalid overlap keyword");
    if (idxs && idx_bytes != 4 && idx_bytes != 8) return fail(CBC_ERR_INVALID, "idx_bytes must be 4 or 8");
    if (!idxs && n_lines > 0 && n_frames != 1 && n_frames != n_lines)
        return fail(CBC_ERR_INVALID, "idxs has an incompatible size (" + std::to_string(n_lines) +
                                         " != " + std::to_string(n_frames) + ")");
    if (n_lines > INT_MAX) return fail(CBC_ERR_INVALID, "too many lines");
    if (D * H * W > INT_MAX) return fail(CBC_ERR_INVALID, "volumes larger than 2^31 voxels");
    if (ck_capacity < 0 || ck_capacity > INT_MAX)
        return fail(CBC_ERR_INVALID, "checkpoint_capacity out of range");
    const long long voxels = n_frames * D * H * W;
    if (n_lines > 0 && voxels > 0 && (!out || !lines)) return fail(CBC_ERR_INVALID, "null pointer");
    const Layout3 L = layout3(n_lines, 0, ck_capacity, 0, sizeof(T));
    if (!workspace || ws_bytes < L.total)
        return fail(CBC_ERR_INVALID, "workspace too small (" + std::to_string(ws_bytes) + " < " +
                                         std::to_string(L.total) + ")");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    init_status_kernel<<<1, 1, 0, s>>>(reinterpret_cast<DevStatus *>(ws + L.status),
                                       CBC_STRATEGY_LINES);
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (n_lines == 0 || voxels == 0) return CBC_OK;
    return run3<T>(out, n_frames, D, H, W, lines, n_lines, idxs, idx_bytes, max_val, kernel,
                   overlap == CBC_MAX ? 1 : 0, ws, L, ck_capacity, 0, nullptr, nullptr, s);
}

template <typename T>
int accumulate3_impl(T *out, long long n_frames, long long D, long long H, long long W,
                     const T *lines, long long n_lines, const void *terms, int term_bytes,
                     const void *frames, int frame_bytes, long long n_terms, T max_val,
                     int kernel, int in_overlap, int out_overlap, void *workspace,
                     size_t ws_bytes, long long ck_capacity, long long table_capacity,
                     void *stream)
{
    clear_error();
    if (n_frames < 0 || D < 0 || H < 0 || W < 0 || n_lines < 0 || n_terms < 0)
        return fail(CBC_ERR_INVALID, "negative size");
    if (kernel < CBC_BIWEIGHT || kernel > CBC_TRIANGULAR)
        return fail(CBC_ERR_INVALID, "kernel is missing");
    if ((in_overlap != CBC_SUM && in_overlap != CBC_MAX) ||
        (out_overlap != CBC_SUM && out_overlap != CBC_MAX))
        return fail(CBC_ERR_INVALID, "Invalid overlap keyword");
    if ((term_bytes != 4 && term_bytes != 8) || (frame_bytes != 4 && frame_bytes != 8))
        return fail(CBC_ERR_INVALID, "term_bytes and frame_bytes must be 4 or 8");
    if (n_lines > 0 && (!terms || !lines)) return fail(CBC_ERR_INVALID, "null pointer");
    if (n_terms > 0 && !frames) return fail(CBC_ERR_INVALID, "null pointer");
    if (n_lines > INT_MAX || n_terms > INT_MAX) return fail(CBC_ERR_INVALID, "too many lines or terms");
    if (D * H * W > INT_MAX) return fail(CBC_ERR_INVALID, "volumes larger than 2^31 voxels");
    if (ck_capacity < 0 || ck_capacity > INT_MAX)
        return fail(CBC_ERR_INVALID, "checkpoint_capacity out of range");
    const int acc = (in_overlap == CBC_MAX ? 1 : 0) | (out_overlap == CBC_MAX ? 2 : 0);
    const bool table = acc == kAccMaxSum || acc == kAccSumMax;
    if (table && (table_capacity < 0 || (table_capacity & (table_capacity - 1))))
        return fail(CBC_ERR_INVALID, "table_capacity must be 0 or a power of two");
    if (!table) table_capacity = 0;
    const long long voxels = n_frames * D * H * W;
    if (n_lines > 0 && voxels > 0 && !out) return fail(CBC_ERR_INVALID, "null pointer");
    const Layout3 L = layout3(n_lines, n_terms, ck_capacity, table_capacity, sizeof(T));
    if (!workspace || ws_bytes < L.total)
        return fail(CBC_ERR_INVALID, "workspace too small (" + std::to_string(ws_bytes) + " < " +
                                         std::to_string(L.total) + ")");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    DevStatus *st = reinterpret_cast<DevStatus *>(ws + L.status);
    int *frame_of_line = reinterpret_cast<int *>(ws + L.frame_of_line);
    int *term_of_line = reinterpret_cast<int *>(ws + L.term_of_line);
    int *frame_of_term = reinterpret_cast<int *>(ws + L.frame_of_term);
    init_status_kernel<<<1, 1, 0, s>>>(st, CBC_STRATEGY_LINES);
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = launch_frames_check(frames, frame_bytes, n_terms, n_frames, frame_of_term, st, s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (n_lines == 0 || voxels == 0) return CBC_OK;
    e = launch_term_frames(terms, term_bytes, frame_of_term, n_lines, n_terms, term_of_line,
                           frame_of_line, st, s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    return run3<T>(out, n_frames, D, H, W, lines, n_lines, frame_of_line, 4, max_val, kernel,
                   4 + acc, ws, L, ck_capacity, table_capacity, term_of_line, frame_of_term, s,
                   n_terms);
}

/* ---- adjoint: gradient of draw_lines with respect to the 3-D line parameters ----
 * (x0, y0, z0, x1, y1, z1, w), from dL/dI, over exactly the voxel visits the forward
 * makes (no counterpart in the reference).  The visits are replayed by the same
 * (column, quadrant) items as render3_kernel; a voxel the reference visits twice adds
 * its term twice under sum overlap, as the forward adds its value twice.  Max overlap:
 * a winner pass first records each voxel's winner (the smallest line whose exact
 * value equals the forward's result and exceeds the volume before drawing, the line
 * sequential std::max keeps), then the gradient pass gives a voxel's term to its
 * winner once: the winner's first visit claims the voxel by swapping its entry to
 * -2 - line, and a last pass puts the winners back. */

/* per-line constants of the voxel terms: end points as given, rmag = 1 / |p1 - p0|^2,
 * the profile's kappa constants and rw = 1 / w */
template <typename T>
struct GradCoef3 {
    T p0[3], p1[3];
    T rmag, k0, k1, rw;
};

template <typename T, int K>
__device__ __forceinline__ GradCoef3<T> make_grad_coef3(const T *ln, T max_val)
{
    GradCoef3<T> c;
    T mag = T(0);
    #pragma unroll
    for (int i = 0; i < 3; i++) {
        c.p0[i] = ln[i];
        c.p1[i] = ln[3 + i];
        const T t = c.p1[i] - c.p0[i];
        mag += t * t;
    }
    c.rmag = T(1) / mag;
    kappa_consts<T, K>(ln[6], max_val, c.k0, c.k1, c.rw);
    return c;
}

/* g * dv/dtheta of one line at voxel P = (X, Y, Z): v[0..6] for x0, y0, z0, x1, y1, z1,
 * w.  With a = p0 - P and e = p1 - P (exact: an integer minus an end point) and
 * t = e - a, s = -(a . t) / |t|^2; beyond an end q is that end point, inside
 * q - P = (t x c) / |t|^2 with c = a x e (each component a difference of products with
 * its FMA error term), so q - P carries no cancellation error, and d^2 = |c|^2 / |t|^2. */
template <typename T, int K>
__device__ __forceinline__ void voxel_term(const GradCoef3<T> &c, T g, const int32_t *P,
                                           T (&v)[7])
{
    T a[3], e[3], t[3];
    #pragma unroll
    for (int i = 0; i < 3; i++) {
        a[i] = c.p0[i] - (T)P[i];
        e[i] = c.p1[i] - (T)P[i];
        t[i] = e[i] - a[i];
    }
    T s = -(a[0] * t[0] + a[1] * t[1] + a[2] * t[2]) * c.rmag;
    T dv[3], d2;
    if (s <= T(0)) {
        s = T(0);
        #pragma unroll
        for (int i = 0; i < 3; i++) dv[i] = a[i];
        d2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    } else if (s >= T(1)) {
        s = T(1);
        #pragma unroll
        for (int i = 0; i < 3; i++) dv[i] = e[i];
        d2 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
    } else {
        const T cx = diff_of_products(a[1], e[2], a[2], e[1]);
        const T cy = diff_of_products(a[2], e[0], a[0], e[2]);
        const T cz = diff_of_products(a[0], e[1], a[1], e[0]);
        dv[0] = (t[1] * cz - t[2] * cy) * c.rmag;
        dv[1] = (t[2] * cx - t[0] * cz) * c.rmag;
        dv[2] = (t[0] * cy - t[1] * cx) * c.rmag;
        d2 = (cx * cx + cy * cy + cz * cz) * c.rmag;
    }
    const T G = g * kappa_d2<T, K>(d2, c.k0, c.k1);
    const T gb = G * s, ga = G - gb;
    #pragma unroll
    for (int i = 0; i < 3; i++) {
        v[i] = ga * dv[i];
        v[3 + i] = gb * dv[i];
    }
    v[6] = -G * d2 * c.rw;
}

/* winner pass: every drawn voxel whose value is the forward's result and above the
 * volume before drawing offers its line; the smallest index stays */
template <typename T, int K>
struct WinnerEmit3 {
    const T *image;
    const T *out0;       /* NULL: zeros */
    int *winner;
    T max_val;
    __device__ __forceinline__ void operator()(long long fbase, long long vox, int line,
                                               T E) const {
        using A = Ar<T>;
        const long long at = fbase + vox;
        const T v = A::mul(max_val, A::template profile<K>(A::sqrt(E)));
        const T img = image[at];
        const T o = out0 ? out0[at] : T(0);
        if (v == img && o < img) atomicMin(winner + at, line);
    }
};

/* gradient pass: the item's terms summed in registers (acc) */
template <typename T, int K, bool MAX>
struct AdjEmit3 {
    const T *grad_out;
    int *winner;         /* MAX: the winner map, claimed entry by entry */
    GradCoef3<T> coef;   /* the current item's line */
    mutable T acc[7];
    __device__ __forceinline__ void voxel(long long fbase, long long vox, int line, T,
                                          const int32_t *cur) const {
        const long long at = fbase + vox;
        if constexpr (MAX) {
            if (winner[at] != line) return;
            if (atomicCAS(winner + at, line, -2 - line) != line) return;   /* counted once */
        }
        const T g = grad_out[at];
        if (g == T(0)) return;
        T v[7];
        voxel_term<T, K>(coef, g, cur, v);
        #pragma unroll
        for (int k = 0; k < 7; k++) acc[k] += v[k];
    }
};

template <typename T>
struct Adj3Args {
    const Rec3<T> *recs;
    const Ck3<T> *cks;
    const T *lines;      /* (N, 7) as given */
    Vol v;
    DevStatus *st;
    double *gacc;        /* (N, 7) */
    T max_val;
};

template <typename T, int K>
__global__ void __launch_bounds__(kThreads)
winner3_kernel(Adj3Args<T> a, WinnerEmit3<T, K> emit)
{
    if (a.st->flags & kFatal) return;
    const long long ncks = (long long)a.st->cks, total = 4 * ncks;
    for (long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x; item < total;
         item += (long long)gridDim.x * blockDim.x) {
        const int q = (int)(item / ncks);
        const Ck3<T> ck = a.cks[item - (long long)q * ncks];
        if (ck.cur[0] == INT_MIN) continue;
        const Rec3<T> r = a.recs[ck.line];
        const long long fbase = (long long)r.frame * a.v.D * a.v.H * a.v.W;
        draw_quadrants(r, column_iter(r, ck), q, q + 1, a.v, fbase, ck.line, emit, a.st);
    }
}

/* one thread per (column, quadrant) as render3_kernel, in warp-uniform steps so that
 * the lanes holding the same line (neighbouring columns) sum their terms by shuffles
 * and one of them adds them to the line's double accumulators */
template <typename T, int K, bool MAX>
__global__ void __launch_bounds__(kThreads)
adjoint3_kernel(Adj3Args<T> a, const T *grad_out, int *winner)
{
    if (a.st->flags & kFatal) return;
    const int lane = threadIdx.x & 31;
    const long long ncks = (long long)a.st->cks, total = 4 * ncks;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
         base < total; base += stride) {
        const long long item = base + lane;
        AdjEmit3<T, K, MAX> em;
        em.grad_out = grad_out;
        em.winner = winner;
        #pragma unroll
        for (int k = 0; k < 7; k++) em.acc[k] = T(0);
        int key = -1;
        if (item < total) {
            const int q = (int)(item / ncks);
            const Ck3<T> ck = a.cks[item - (long long)q * ncks];
            if (ck.cur[0] != INT_MIN) {
                const Rec3<T> r = a.recs[ck.line];
                key = ck.line;
                em.coef = make_grad_coef3<T, K>(a.lines + (size_t)ck.line * 7, a.max_val);
                const long long fbase = (long long)r.frame * a.v.D * a.v.H * a.v.W;
                draw_quadrants(r, column_iter(r, ck), q, q + 1, a.v, fbase, ck.line, em, a.st);
            }
        }
        __syncwarp();
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(peers) - 1;
        const int most = __reduce_max_sync(0xffffffffu, key >= 0 ? __popc(peers) : 0);
        T sum[7];
        #pragma unroll
        for (int k = 0; k < 7; k++) sum[k] = em.acc[k];
        unsigned rest = peers & (peers - 1u);            /* the group without its leader */
        for (int i = 1; i < most; i++) {
            const int src = rest ? __ffs(rest) - 1 : lane;
            const bool take = lane == leader && rest != 0u;
            #pragma unroll
            for (int k = 0; k < 7; k++) {
                const T o = __shfl_sync(0xffffffffu, em.acc[k], src);
                if (take) sum[k] += o;
            }
            rest &= rest - 1u;
        }
        if (key >= 0 && lane == leader) {
            #pragma unroll
            for (int k = 0; k < 7; k++)
                if (sum[k] != T(0)) atomicAdd(a.gacc + (size_t)key * 7 + k, (double)sum[k]);
        }
    }
}

/* the double sums into grad_lines; claimed winners (-2 - line) back to their lines */
template <typename T>
__global__ void __launch_bounds__(kThreads)
adjoint3_finish_kernel(const double *__restrict__ gacc, T *__restrict__ grad, long long n7,
                       int *__restrict__ winner, long long n_vox)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n7; i += stride)
        grad[i] = (T)gacc[i];
    if (!winner) return;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_vox; i += stride) {
        const int w = winner[i];
        if (w < -1) winner[i] = -2 - w;
    }
}

/* workspace of the 3-D adjoint: the draw layout, then the (N, 7) double sums */
inline size_t adjoint3_gacc_offset(long long n_lines, long long ck_capacity, size_t elem)
{
    return layout3(n_lines, 0, ck_capacity, 0, elem).total;
}

inline size_t adjoint3_workspace(long long n_lines, long long ck_capacity, size_t elem)
{
    return adjoint3_gacc_offset(n_lines, ck_capacity, elem) +
           ((sizeof(double) * 7 * (size_t)n_lines + 255) / 256) * 256;
}

template <typename T, int K>
cudaError_t launch_adjoint3(const Adj3Args<T> &a, int overlap, const T *grad_out,
                            const T *image, const T *out0, int *winner, cudaStream_t s)
{
    if (overlap == CBC_MAX) {
        WinnerEmit3<T, K> we{image, out0, winner, a.max_val};
        winner3_kernel<T, K><<<resident_grid(winner3_kernel<T, K>, kThreads), kThreads, 0, s>>>(
            a, we);
        adjoint3_kernel<T, K, true>
            <<<resident_grid(adjoint3_kernel<T, K, true>, kThreads), kThreads, 0, s>>>(
                a, grad_out, winner);
        note_launches(2);
    } else {
        adjoint3_kernel<T, K, false>
            <<<resident_grid(adjoint3_kernel<T, K, false>, kThreads), kThreads, 0, s>>>(
                a, grad_out, nullptr);
        note_launches(1);
    }
    return cudaGetLastError();
}

template <typename T>
int backward3_impl(const T *grad_out, long long n_frames, long long D, long long H, long long W,
                   const T *lines, long long n_lines, const void *idxs, int idx_bytes,
                   T max_val, int kernel, int overlap, const T *image, const T *out0,
                   int *winner, T *grad_lines, void *workspace, size_t ws_bytes,
                   long long ck_capacity, void *stream)
{
    clear_error();
    if (n_frames < 0 || D < 0 || H < 0 || W < 0 || n_lines < 0)
        return fail(CBC_ERR_INVALID, "negative size");
    if (kernel < CBC_BIWEIGHT || kernel > CBC_TRIANGULAR)
        return fail(CBC_ERR_INVALID, "kernel is missing");
    if (overlap != CBC_SUM && overlap != CBC_MAX) return fail(CBC_ERR_INVALID, "Invalid overlap keyword");
    if (idxs && idx_bytes != 4 && idx_bytes != 8) return fail(CBC_ERR_INVALID, "idx_bytes must be 4 or 8");
    if (!idxs && n_lines > 0 && n_frames != 1 && n_frames != n_lines)
        return fail(CBC_ERR_INVALID, "idxs has an incompatible size (" + std::to_string(n_lines) +
                                         " != " + std::to_string(n_frames) + ")");
    if (n_lines > INT_MAX) return fail(CBC_ERR_INVALID, "too many lines");
    if (D * H * W > INT_MAX) return fail(CBC_ERR_INVALID, "volumes larger than 2^31 voxels");
    if (ck_capacity < 0 || ck_capacity > INT_MAX)
        return fail(CBC_ERR_INVALID, "checkpoint_capacity out of range");
    const long long voxels = n_frames * D * H * W;
    if (n_lines > 0 && (!lines || !grad_lines)) return fail(CBC_ERR_INVALID, "null pointer");
    if (n_lines > 0 && voxels > 0 && !grad_out) return fail(CBC_ERR_INVALID, "null pointer");
    if (overlap == CBC_MAX && n_lines > 0 && voxels > 0 && (!image || !winner))
        return fail(CBC_ERR_INVALID, "max overlap needs the forward image and a winner buffer");
    const Layout3 L = layout3(n_lines, 0, ck_capacity, 0, sizeof(T));
    const size_t need = adjoint3_workspace(n_lines, ck_capacity, sizeof(T));
    if (!workspace || ws_bytes < need)
        return fail(CBC_ERR_INVALID, "workspace too small (" + std::to_string(ws_bytes) + " < " +
                                         std::to_string(need) + ")");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    DevStatus *st = reinterpret_cast<DevStatus *>(ws + L.status);
    double *gacc = reinterpret_cast<double *>(ws + adjoint3_gacc_offset(n_lines, ck_capacity,
                                                                        sizeof(T)));
    init_status_kernel<<<1, 1, 0, s>>>(st, CBC_STRATEGY_LINES);
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && n_lines > 0)
        e = cudaMemsetAsync(gacc, 0, sizeof(double) * 7 * (size_t)n_lines, s);
    const bool maxw = overlap == CBC_MAX && voxels > 0 && n_lines > 0;
    if (e == cudaSuccess && maxw)
        e = cudaMemsetAsync(winner, 0x7f, sizeof(int) * (size_t)voxels, s);   /* no winner */
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (n_lines == 0) return CBC_OK;
    if (voxels > 0) {
        Rec3<T> *recs = reinterpret_cast<Rec3<T> *>(ws + L.recs);
        Ck3<T> *cks = reinterpret_cast<Ck3<T> *>(ws + L.cks);
        Vol v{(int)D, (int)H, (int)W};
        const unsigned nb = (unsigned)((n_lines + kThreads - 1) / kThreads);
        if (idxs && idx_bytes == 8)
            prep3_kernel<T, int64_t><<<nb, kThreads, 0, s>>>(lines, idxs, n_lines, n_frames, v,
                                                             recs, cks, ck_capacity, st);
        else
            prep3_kernel<T, int32_t><<<nb, kThreads, 0, s>>>(lines, idxs, n_lines, n_frames, v,
                                                             recs, cks, ck_capacity, st);
        note_launches(1);
        Adj3Args<T> a{recs, cks, lines, v, st, gacc, max_val};
        switch (kernel) {
        case CBC_BIWEIGHT:    e = launch_adjoint3<T, CBC_BIWEIGHT>(a, overlap, grad_out, image, out0, winner, s); break;
        case CBC_GAUSSIAN:    e = launch_adjoint3<T, CBC_GAUSSIAN>(a, overlap, grad_out, image, out0, winner, s); break;
        case CBC_PARABOLIC:   e = launch_adjoint3<T, CBC_PARABOLIC>(a, overlap, grad_out, image, out0, winner, s); break;
        case CBC_RECTANGULAR: e = launch_adjoint3<T, CBC_RECTANGULAR>(a, overlap, grad_out, image, out0, winner, s); break;
        default:              e = launch_adjoint3<T, CBC_TRIANGULAR>(a, overlap, grad_out, image, out0, winner, s); break;
        }
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    }
    const long long n7 = 7 * n_lines;
    const long long work = maxw && voxels > n7 ? voxels : n7;
    long long blocks = (work + kThreads - 1) / kThreads;
    if (blocks > 4096) blocks = 4096;
    adjoint3_finish_kernel<T><<<(unsigned)blocks, kThreads, 0, s>>>(gacc, grad_lines, n7,
                                                                    maxw ? winner : nullptr,
                                                                    voxels);
    note_launches(1);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    return CBC_OK;
}

}  // namespace l3
}  // namespace cbc

extern "C" {

size_t cbc_draw_lines_3d_workspace_size(int64_t n_lines, int64_t checkpoint_capacity,
                                        int32_t elem_bytes)
{
    if (n_lines < 0 || checkpoint_capacity < 0 || (elem_bytes != 4 && elem_bytes != 8)) return 0;
    return cbc::l3::layout3(n_lines, 0, checkpoint_capacity, 0, (size_t)elem_bytes).total;
}

int cbc_draw_lines_3d_f32(float *out, int64_t n_frames, int64_t depth, int64_t height,
                          int64_t width, const float *lines, int64_t n_lines, const void *idxs,
                          int32_t idx_bytes, float max_val, int32_t kernel, int32_t overlap,
                          void *workspace, size_t workspace_bytes, int64_t checkpoint_capacity,
                          void *stream)
{
    return cbc::l3::draw3_impl<float>(out, n_frames, depth, height, width, lines, n_lines, idxs,
                                      idx_bytes, max_val, kernel, overlap, workspace,
                                      workspace_bytes, checkpoint_capacity, stream);
}

int cbc_draw_lines_3d_f64(double *out, int64_t n_frames, int64_t depth, int64_t height,
                          int64_t width, const double *lines, int64_t n_lines, const void *idxs,
                          int32_t idx_bytes, double max_val, int32_t kernel, int32_t overlap,
                          void *workspace, size_t workspace_bytes, int64_t checkpoint_capacity,
                          void *stream)
{
    return cbc::l3::draw3_impl<double>(out, n_frames, depth, height, width, lines, n_lines, idxs,
                                       idx_bytes, max_val, kernel, overlap, workspace,
                                       workspace_bytes, checkpoint_capacity, stream);
}

size_t cbc_accumulate_lines_3d_workspace_size(int64_t n_lines, int64_t n_terms,
                                              int64_t checkpoint_capacity,
                                              int64_t table_capacity, int32_t elem_bytes)
{
    if (n_lines < 0 || n_terms < 0 || checkpoint_capacity < 0 || table_capacity < 0 ||
        (elem_bytes != 4 && elem_bytes != 8))
        return 0;
    return cbc::l3::layout3(n_lines, n_terms, checkpoint_capacity, table_capacity,
                            (size_t)elem_bytes).total;
}

int cbc_accumulate_lines_3d_f32(float *out, int64_t n_frames, int64_t depth, int64_t height,
                                int64_t width, const float *lines, int64_t n_lines,
                                const void *terms, int32_t term_bytes, const void *frames,
                                int32_t frame_bytes, int64_t n_terms, float max_val,
                                int32_t kernel, int32_t in_overlap, int32_t out_overlap,
                                void *workspace, size_t workspace_bytes,
                                int64_t checkpoint_capacity, int64_t table_capacity, void *stream)
{
    return cbc::l3::accumulate3_impl<float>(out, n_frames, depth, height, width, lines, n_lines,
                                            terms, term_bytes, frames, frame_bytes, n_terms,
                                            max_val, kernel, in_overlap, out_overlap, workspace,
                                            workspace_bytes, checkpoint_capacity, table_capacity,
                                            stream);
}

int cbc_accumulate_lines_3d_f64(double *out, int64_t n_frames, int64_t depth, int64_t height,
                                int64_t width, const double *lines, int64_t n_lines,
                                const void *terms, int32_t term_bytes, const void *frames,
                                int32_t frame_bytes, int64_t n_terms, double max_val,
                                int32_t kernel, int32_t in_overlap, int32_t out_overlap,
                                void *workspace, size_t workspace_bytes,
                                int64_t checkpoint_capacity, int64_t table_capacity, void *stream)
{
    return cbc::l3::accumulate3_impl<double>(out, n_frames, depth, height, width, lines, n_lines,
                                             terms, term_bytes, frames, frame_bytes, n_terms,
                                             max_val, kernel, in_overlap, out_overlap, workspace,
                                             workspace_bytes, checkpoint_capacity,
                                             table_capacity, stream);
}

size_t cbc_draw_lines_3d_backward_workspace_size(int64_t n_lines, int64_t checkpoint_capacity,
                                                 int32_t elem_bytes)
{
    if (n_lines < 0 || checkpoint_capacity < 0 || (elem_bytes != 4 && elem_bytes != 8)) return 0;
    return cbc::l3::adjoint3_workspace(n_lines, checkpoint_capacity, (size_t)elem_bytes);
}

int cbc_draw_lines_3d_backward_f32(const float *grad_out, int64_t n_frames, int64_t depth,
                                   int64_t height, int64_t width, const float *lines,
                                   int64_t n_lines, const void *idxs, int32_t idx_bytes,
                                   float max_val, int32_t kernel, int32_t overlap,
                                   const float *image, const float *out0, int32_t *winner,
                                   float *grad_lines, void *workspace, size_t workspace_bytes,
                                   int64_t checkpoint_capacity, void *stream)
{
    return cbc::l3::backward3_impl<float>(grad_out, n_frames, depth, height, width, lines,
                                          n_lines, idxs, idx_bytes, max_val, kernel, overlap,
                                          image, out0, winner, grad_lines, workspace,
                                          workspace_bytes, checkpoint_capacity, stream);
}

int cbc_draw_lines_3d_backward_f64(const double *grad_out, int64_t n_frames, int64_t depth,
                                   int64_t height, int64_t width, const double *lines,
                                   int64_t n_lines, const void *idxs, int32_t idx_bytes,
                                   double max_val, int32_t kernel, int32_t overlap,
                                   const double *image, const double *out0, int32_t *winner,
                                   double *grad_lines, void *workspace, size_t workspace_bytes,
                                   int64_t checkpoint_capacity, void *stream)
{
    return cbc::l3::backward3_impl<double>(grad_out, n_frames, depth, height, width, lines,
                                           n_lines, idxs, idx_bytes, max_val, kernel, overlap,
                                           image, out0, winner, grad_lines, workspace,
                                           workspace_bytes, checkpoint_capacity, stream);
}

}  // extern "C"
