/*
 * cbc_adjoint.cu — gradient of draw_lines with respect to the line parameters (no
 * counterpart in the reference, which differentiates only its geometry).
 *
 * A line draws v = max_val * K(x), x = d / w, at every pixel its walk draws, d being
 * the distance from the pixel to the segment (the walk's error E is (d / w)^2 in exact
 * arithmetic, bresenham.hpp:291-296).  With q = p0 + s (p1 - p0) the nearest point of
 * the segment (s clamped to [0, 1]) the envelope theorem gives
 *     dv/dp0 = kappa (1 - s) (q - p),  dv/dp1 = kappa s (q - p),  dv/dw = -kappa d^2 / w
 * with kappa = max_val K'(x) / (d w), which is finite at d = 0 for the smooth profiles
 * (biweight -3.75 (1 - x^2) / w^2, gaussian -9 K(x) / w^2, parabolic -1.5 / w^2;
 * rectangular 0; triangular -1 / (d w), taken as 0 at d = 0).
 *
 * The pixels are exactly the forward's.  Sum overlap: drive_segments (cbc_common.cuh)
 * enumerates every line's walk again with the reference's arithmetic and adds each
 * drawn pixel's term; per-line sums are kept per segment in shared memory, then in
 * double in global memory.  Max overlap: a pixel's gradient goes to one line, the
 * smallest line index whose exact value equals the final pixel value (and exceeds the
 * value before drawing; sequential std::max keeps the first such line).  Those
 * winners come from the forward (cbc_draw_lines_max_winner_f32) or from a walk pass
 * that recomputes them, and the gradient is then one streaming pass over the pixels
 * (dense_max_kernel) that adds each pixel's term to its winner's sums.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <limits.h>
#include <cmath>
#include <string>

#include "cbc_common.cuh"

namespace cbc {


/* max overlap: winner[p] = min over lines l with v_l(p) == image[p] > out0[p] */
template <typename T, int K>
struct WinnerAct {
    static constexpr bool kNeedsError = true;
    const T *image;
    const T *out0;       /* NULL: zeros */
    int *winner;
    T max_val;
    int W;
    const float *gtab;   /* gaussian table (shared-memory copy) */
    struct Pre {
        T img, o;
    };
    template <class ST>
    __device__ __forceinline__ void item_begin(int, const ST &) {}
    __device__ __forceinline__ void item_end(int, const SlotTable<T> &) {}
    __device__ __forceinline__ Pre prefetch(const SlotTable<T> &S, int slot, int px, int py) const {
        const long long at = S.fbase[slot] + (long long)py * W + px;
        Pre p;
        p.img = image[at];
        p.o = out0 ? out0[at] : T(0);
        return p;
    }
    __device__ __forceinline__ void pixel(const SlotTable<T> &S, int slot, int px, int py, T E,
                                          T, T, const Pre &p) {
        using A = Ar<T>;
        const long long at = S.fbase[slot] + (long long)py * W + px;
        const T v = A::mul(max_val, A::template profile_tab<K>(A::sqrt(E), gtab));
        if (v == p.img && p.o < p.img) atomicMin(winner + at, S.line[slot]);
    }
};

/* per-line constants of the pixel terms: the segment's end points p0 = (x0, y0) and
 * p1 = (x1, y1) as given, rmag = 1 / |p1 - p0|^2, and kappa(d^2) = k0 + k1 d^2
 * (biweight, parabolic), k0 exp(k1 d^2) (gaussian), k0 / d (triangular, 0 at d = 0)
 * or 0 (rectangular); rw = 1 / w. */
template <typename T>
struct alignas(8 * sizeof(T)) GradCoef {
    T x0, y0, x1, y1, rmag, k0, k1, rw;
};

/* the constants of a line from its end points and width */
template <typename T, int K>
__device__ __forceinline__ GradCoef<T> make_grad_coef(T x0, T y0, T x1, T y1, T w, T max_val)
{
    GradCoef<T> c;
    c.x0 = x0;
    c.y0 = y0;
    c.x1 = x1;
    c.y1 = y1;
    const T t0 = x1 - x0, t1 = y1 - y0;
    c.rmag = T(1) / (t0 * t0 + t1 * t1);
    kappa_consts<T, K>(w, max_val, c.k0, c.k1, c.rw);
    return c;
}

template <typename T, int K>
__global__ void __launch_bounds__(256)
grad_coef_kernel(const T *__restrict__ lines, long long n, T max_val,
                 GradCoef<T> *__restrict__ coef)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const T *ln = lines + i * 5;
    coef[i] = make_grad_coef<T, K>(ln[0], ln[1], ln[2], ln[3], ln[4], max_val);
}

/* g * dv/dtheta of one line at pixel (X, Y): v[0..4] for x0, y0, x1, y1, w.
 * The geometry is taken relative to the pixel from the end points as given: a pixel
 * coordinate (an integer) minus an end point is exact in T whenever the difference
 * is below 2^p ulp(end point), so q - P has no cancellation error.  Inside the
 * segment's extent (0 < s < 1) q - P = c (t1, -t0) rmag with c = (p0 - P) x (p1 - P),
 * evaluated as a difference of products with an FMA error term (within 2 ulp of the
 * exact cross product); beyond an end q is that end point.  s itself only weights the
 * two end points, so its rounding does not cancel. */
template <typename T, int K>
__device__ __forceinline__ void pixel_term(const GradCoef<T> &c, T g, T X, T Y, T (&v)[5])
{
    const T a = c.x0 - X, b = c.y0 - Y, e = c.x1 - X, f = c.y1 - Y;
    const T t0 = e - a, t1 = f - b;
    T s = -(a * t0 + b * t1) * c.rmag;
    T dx, dy, d2;
    if (s <= T(0)) {
        s = T(0);
        dx = a;
        dy = b;
        d2 = a * a + b * b;
    } else if (s >= T(1)) {
        s = T(1);
        dx = e;
        dy = f;
        d2 = e * e + f * f;
    } else {
        const T be = b * e;
        const T cr = fma_rn(a, f, -be) + fma_rn(-b, e, be);
        const T u = cr * c.rmag;
        dx = u * t1;
        dy = -u * t0;
        d2 = cr * u;
    }
    const T G = g * kappa_d2<T, K>(d2, c.k0, c.k1);
    const T gb = G * s, ga = G - gb;
    v[0] = ga * dx;
    v[1] = ga * dy;
    v[2] = gb * dx;
    v[3] = gb * dy;
    v[4] = -G * d2 * c.rw;
}

/* sum overlap: every drawn pixel (error <= 1) of every line gets its term */
template <typename T, int K>
struct BackwardAct {
    static constexpr bool kNeedsError = true;
    const T *lines;      /* (N, 5) parameters as given */
    const T *grad_out;   /* dL/dI, or NULL with image and target: L = sum((I - T)^2) */
    const T *image;
    const T *target;
    double *gacc;        /* (N, 5) */
    T (*acc)[5];         /* this warp's per-slot accumulators (shared memory) */
    GradCoef<T> *coef;   /* this warp's per-slot term constants (shared memory) */
    T max_val;
    int W;
    __device__ __forceinline__ void item_begin(int lane, const SlotTable<T> &S) {
        #pragma unroll
        for (int k = 0; k < 5; k++) acc[lane][k] = T(0);
        const int line = S.line[lane];
        if (line >= 0) {
            const T *ln = lines + (size_t)line * 5;
            coef[lane] = make_grad_coef<T, K>(ln[0], ln[1], ln[2], ln[3], ln[4], max_val);
        }
    }
    __device__ __forceinline__ void item_end(int lane, const SlotTable<T> &S) {
        const int line = S.line[lane];
        if (line < 0) return;
        #pragma unroll
        for (int k = 0; k < 5; k++) {
            const T v = acc[lane][k];
            if (v != T(0)) atomicAdd(gacc + (size_t)line * 5 + k, (double)v);
        }
    }
    struct Pre {
        T g;
    };
    __device__ __forceinline__ Pre prefetch(const SlotTable<T> &S, int slot, int px, int py) const {
        const long long at = S.fbase[slot] + (long long)py * W + px;
        Pre p;
        p.g = grad_out ? grad_out[at] : T(2) * (image[at] - target[at]);
        return p;
    }
    /* this lane's term of the current drain batch, added in batch_end */
    T pv[5];
    int pslot = -1;
    __device__ __forceinline__ void pixel(const SlotTable<T> &S, int slot, int px, int py, T, T,
                                          T, const Pre &p) {
        const T g = p.g;
        if (g == T(0)) return;
        pixel_term<T, K>(coef[slot], g, (T)px, (T)py, pv);
        pslot = slot;
    }
    /* the batch's terms into the per-slot sums: lanes holding the same slot (the lanes
     * of one drain batch often do) are summed by shuffles into their lowest lane, which
     * alone adds to the slot, so the sums need no shared-memory atomics */
    __device__ __forceinline__ void batch_end(int lane) {
        const int key = pslot;
        if (__ballot_sync(0xffffffffu, key >= 0) == 0u) return;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(peers) - 1;
        const int most = __reduce_max_sync(0xffffffffu, key >= 0 ? __popc(peers) : 0);
        T s[5];
        #pragma unroll
        for (int k = 0; k < 5; k++) s[k] = pv[k];
        unsigned rest = peers & (peers - 1u);            /* the group without its leader */
        for (int r = 1; r < most; r++) {
            const int src = rest ? __ffs(rest) - 1 : lane;
            const bool take = lane == leader && rest != 0u;
            #pragma unroll
            for (int k = 0; k < 5; k++) {
                const T o = __shfl_sync(0xffffffffu, pv[k], src);
                if (take) s[k] += o;
            }
            rest &= rest - 1u;
        }
        if (key >= 0 && lane == leader) {
            #pragma unroll
            for (int k = 0; k < 5; k++)
                if (s[k] != T(0)) acc[key][k] += s[k];
        }
        pslot = -1;
    }
};

/* ---- max overlap: the adjoint as one pass over the pixels ----
 * Under max overlap a drawn pixel's value comes from one line, its winner, so its
 * adjoint is one line's term.  Rather than walking every line again and testing each
 * pixel's winner, the pass streams the winners (or the forward's packed (value,
 * winner) words) and dL/dI over the frames once, with 16-byte loads, and adds each
 * drawn pixel's term to its winner's sums.
 *
 * The frames are read as a flat array of 8-pixel chunks.  A thread takes a patch of
 * kPatchRows chunks one pitch apart, the pitch being W / 8 chunks rounded, so the
 * chunks of a patch lie one below the other (sheared by at most 4 pixels per row) and
 * neighbouring threads read neighbouring chunks.  A chunk row of a warp (32 chunks)
 * has ~40 % drawn pixels, so rather than evaluating its 256 pixel positions with most
 * lanes idle the warp compacts the drawn ones into a shared-memory queue and each lane
 * evaluates a contiguous run of about total / 32 of them.  A lane keeps the sums of
 * the two lines it met last in registers and flushes a line's sums to the double
 * accumulators only when it makes room for another line, so a line reaches global
 * memory a few times per patch row rather than once per pixel.  The per-line
 * constants come from a table that one thread per line fills first
 * (grad_coef_kernel). */
constexpr int kChunk = 8;
constexpr int kPatchRows = 8;
constexpr int kDenseThreads = 256;

enum : int { kSrcPacked = 0, kSrcWinner = 1 };

template <typename T>
struct DenseArgs {
    const unsigned long long *packed;   /* kSrcPacked: (value bits << 32) | ~line, 0: undrawn */
    unsigned long long *clear;          /* kSrcPacked: zero the words after reading, or NULL */
    const int *winner;                  /* kSrcWinner: line index, outside [0, N): none */
    const T *grad_out;                  /* dL/dI, or NULL: 2 (I - target) */
    const T *image;                     /* kSrcWinner without grad_out */
    const T *target;
    const GradCoef<T> *coef;            /* (N) */
    double *gacc;                       /* (N, 5) sums */
    double *partials;                   /* kSrcPacked: per-block sum of I (I - 2 T) over
                                           drawn pixels, or NULL */
    const DevStatus *st;                /* the forward's status (fatal: no gradient), or NULL */
    int *err;                           /* status flags to mark a wait that gave up */
    unsigned long long *tasks;          /* task counter, zero at launch */
    long long n_px, n_chunks, n_items;
    long long n_full;                   /* chunks of kChunk pixels wholly inside the frames */
    int n_lines, H, W, pitch;
    int vec;                            /* every base pointer is 16-byte aligned */
    int tma;                            /* the tensor maps of the packed words and targets
                                           are valid (kSrcPacked) */
};

/* 8 elements from p + p0: two or four 16-byte loads when aligned and in range */
template <typename U>
__device__ __forceinline__ void load_chunk(const U *p, long long p0, long long n, bool vec,
                                           U (&v)[kChunk])
{
    if (vec && p0 + kChunk <= n) {
        constexpr int kQ = kChunk * (int)sizeof(U) / 16;
        uint4 q[kQ];
        const uint4 *src = reinterpret_cast<const uint4 *>(p + p0);
        #pragma unroll
        for (int i = 0; i < kQ; i++) q[i] = src[i];
        __builtin_memcpy(v, q, sizeof(v));
    } else {
        #pragma unroll
        for (int e = 0; e < kChunk; e++) v[e] = p0 + e < n ? p[p0 + e] : U(0);
    }
}

/* a line's running sums with its constants */
template <typename T>
struct GradSlot {
    int id;
    GradCoef<T> c;
    T s[5];
    __device__ __forceinline__ void open(const GradCoef<T> *coef, int line) {
        id = line;
        c = coef[line];
        #pragma unroll
        for (int k = 0; k < 5; k++) s[k] = T(0);
    }
    __device__ __forceinline__ void flush(double *gacc) const {
        if (id < 0) return;
        double *g = gacc + (size_t)id * 5;
        #pragma unroll
        for (int k = 0; k < 5; k++)
            if (s[k] != T(0)) atomicAdd(g + k, (double)s[k]);
    }
};

/* two lines' running sums, the least recently used one making room for a new line */
template <typename T>
struct SlotPair {
    GradSlot<T> A, B;
    bool mru_a;
    template <int K>
    __device__ __forceinline__ void add(const DenseArgs<T> &a, int line, T g, T X, T Y) {
        bool in_a = line == A.id;
        if (!in_a && line != B.id) {
            if (mru_a) {
                B.flush(a.gacc);
                B.open(a.coef, line);
            } else {
                A.flush(a.gacc);
                A.open(a.coef, line);
                in_a = true;
            }
        }
        mru_a = in_a;
        GradCoef<T> c;
        c.x0 = in_a ? A.c.x0 : B.c.x0;
        c.y0 = in_a ? A.c.y0 : B.c.y0;
        c.x1 = in_a ? A.c.x1 : B.c.x1;
        c.y1 = in_a ? A.c.y1 : B.c.y1;
        c.rmag = in_a ? A.c.rmag : B.c.rmag;
        c.k0 = in_a ? A.c.k0 : B.c.k0;
        c.k1 = in_a ? A.c.k1 : B.c.k1;
        c.rw = in_a ? A.c.rw : B.c.rw;
        T v[5];
        pixel_term<T, K>(c, g, X, Y, v);
        #pragma unroll
        for (int k = 0; k < 5; k++) {
            if (in_a) A.s[k] += v[k];
            else B.s[k] += v[k];
        }
    }
};

/* advance pixel coordinates (x, y) by n >= 0 pixels of a W x H frame */
__device__ __forceinline__ void advance_px(int &x, int &y, int n, int W, int H)
{
    x += n;
    while (x >= W) {
        x -= W;
        if (++y == H) y = 0;
    }
}

/* the per-warp queue of one chunk row's drawn pixels (up to 32 x 8), padded by one
 * entry per 32 so that lane l reading entry l * m + r hits distinct banks */
constexpr int kDenseWarps = kDenseThreads / 32;
constexpr int kQueue = 32 * kChunk + kChunk;
constexpr int kDenseMaxBlocks = 2048;   /* persistent grid cap = loss partials */

__device__ __forceinline__ int qslot(int i) { return i + (i >> 5); }

/* ---- staging of the packed pass ----
 * A warp's chunk row is 32 chunks of 8 pixels: 2 KB of packed words and 1 KB of
 * targets.  Where the 32 chunks are consecutive and whole (most rows: they are unless
 * the row straddles a band edge or reaches the end of the frames) the row is fetched
 * by the tensor memory accelerator: two cp.async.bulk.tensor copies issued by lane 0
 * (boxes of 32 chunks x 64 B and 32 chunks x 32 B) that complete on the buffer's
 * mbarrier, with the 64 B / 32 B swizzle so that each lane's 16-byte reads of its own
 * chunk hit distinct banks.  Other rows are loaded by the lanes into the same swizzled
 * layout.  Two buffers per warp: row k + 1 is in flight while row k is evaluated. */
constexpr int kPkPieces = kChunk * 8 / 16;      /* 16-byte pieces of a chunk's packed words */
constexpr int kTgPieces = kChunk * 4 / 16;      /* ... of its targets                       */
constexpr int kPkRow = 32 * kChunk * 8;         /* bytes of a warp's row of packed words    */
constexpr int kTgRow = 32 * kChunk * 4;         /* ... of targets                           */
constexpr int kStageAlign = 1024;               /* the swizzle patterns repeat within this  */
constexpr long long kWaitLimit = 1ll << 22;     /* bounded mbarrier waits (try_wait rounds) */

struct PackedStage {
    unsigned char pk[kDenseWarps][2][kPkRow];
    unsigned char tg[kDenseWarps][2][kTgRow];
    unsigned long long bar[kDenseWarps][2];      /* mbarriers of the TMA buffers */
};

template <typename T>
struct DenseQueueT {
    int line[kDenseWarps][kQueue];
    T g[kDenseWarps][kQueue];
    unsigned char pos[kDenseWarps][kQueue];
    int x[kDenseWarps][32], y[kDenseWarps][32];
};

template <typename T>
__host__ __device__ constexpr size_t dense_stage_offset()
{
    return (sizeof(DenseQueueT<T>) + 15) / 16 * 16;
}

template <typename T, int SRC>
constexpr size_t dense_smem()
{
    return SRC == kSrcPacked && sizeof(T) == 4
               ? dense_stage_offset<T>() + kStageAlign + sizeof(PackedStage)
               : sizeof(DenseQueueT<T>);
}

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

/* byte offset of 16-byte piece j of row r in a swizzled row buffer starting at shared
 * address `base` (1024-aligned): rows of 64 B take the 64 B swizzle (piece index XOR
 * address bits 7-8), rows of 32 B the 32 B swizzle (XOR address bit 7) */
template <int ROW>
__device__ __forceinline__ unsigned swz(unsigned base, int r, int j)
{
    const unsigned row = base + (unsigned)r * ROW;
    const unsigned mask = ROW == 64 ? 3u : 1u;
    return (unsigned)r * ROW + 16u * ((unsigned)j ^ ((row >> 7) & mask));
}

__device__ __forceinline__ void mbar_init(unsigned bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned phase)
{
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(phase)
        : "memory");
    return ok != 0;
}

/* lane 0: fetch box {0, c0} of both tensor maps into the buffer, completing on `bar` */
__device__ __forceinline__ void tma_row(unsigned dst_pk, unsigned dst_tg, unsigned bar,
                                        const CUtensorMap *tm_pk, const CUtensorMap *tm_tg,
                                        long long c0)
{
    const int y = (int)c0;
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n"
                 ::"r"(bar), "r"(kPkRow + kTgRow) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];\n"
        ::"r"(dst_pk), "l"(reinterpret_cast<unsigned long long>(tm_pk)), "r"(0), "r"(y),
          "r"(bar) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];\n"
        ::"r"(dst_tg), "l"(reinterpret_cast<unsigned long long>(tm_tg)), "r"(0), "r"(y),
          "r"(bar) : "memory");
}

/* start staging chunk row `cc` (this lane's chunk) into buffer buf: by TMA when the
 * warp's 32 chunks are consecutive and whole, else by the lanes' own loads.  Returns
 * true when a TMA copy is pending on the buffer's mbarrier. */
__device__ __forceinline__ bool stage_row(unsigned char *pk, unsigned char *tg, unsigned bar,
                                          int lane, long long cc, const DenseArgs<float> &a,
                                          const CUtensorMap *tm_pk, const CUtensorMap *tm_tg)
{
    const long long c0 = __shfl_sync(0xffffffffu, cc, 0);
    const bool tma = a.tma && __all_sync(0xffffffffu, cc == c0 + lane) && c0 + 32 <= a.n_full;
    __syncwarp();                        /* every lane is done with the buffer's last row */
    if (tma) {
        if (lane == 0) tma_row(smem_addr(pk), smem_addr(tg), bar, tm_pk, tm_tg, c0);
        return true;
    }
    unsigned long long w[kChunk];
    float t[kChunk];
    const long long p0 = cc * kChunk;
    if (cc < a.n_chunks && a.vec && p0 + kChunk <= a.n_px) {
        const uint4 *gp = reinterpret_cast<const uint4 *>(a.packed + p0);
        const uint4 *gt = reinterpret_cast<const uint4 *>(a.target + p0);
        uint4 q[kPkPieces], r[kTgPieces];
        #pragma unroll
        for (int j = 0; j < kPkPieces; j++) q[j] = gp[j];
        #pragma unroll
        for (int j = 0; j < kTgPieces; j++) r[j] = gt[j];
        __builtin_memcpy(w, q, sizeof(w));
        __builtin_memcpy(t, r, sizeof(t));
    } else {
        #pragma unroll
        for (int e = 0; e < kChunk; e++) {
            const bool in = cc < a.n_chunks && p0 + e < a.n_px;
            w[e] = in ? a.packed[p0 + e] : 0ull;
            t[e] = in ? a.target[p0 + e] : 0.0f;
        }
    }
    uint4 q[kPkPieces], r[kTgPieces];
    __builtin_memcpy(q, w, sizeof(w));
    __builtin_memcpy(r, t, sizeof(t));
    const unsigned bp = smem_addr(pk), bt = smem_addr(tg);
    #pragma unroll
    for (int j = 0; j < kPkPieces; j++)
        *reinterpret_cast<uint4 *>(pk + swz<64>(bp, lane, j)) = q[j];
    #pragma unroll
    for (int j = 0; j < kTgPieces; j++)
        *reinterpret_cast<uint4 *>(tg + swz<32>(bt, lane, j)) = r[j];
    return false;
}

/* Persistent: each warp takes tasks of 32 patches (one per lane) from a counter until
 * none are left, so the warps end together whatever the drawn density. */
template <typename T, int K, int SRC>
__global__ void __launch_bounds__(kDenseThreads, 3)
dense_max_kernel(DenseArgs<T> a, const __grid_constant__ CUtensorMap tm_pk,
                 const __grid_constant__ CUtensorMap tm_tg)
{
    extern __shared__ __align__(16) unsigned char dense_smem_raw[];
    DenseQueueT<T> &Q = *reinterpret_cast<DenseQueueT<T> *>(dense_smem_raw);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    /* the stage at the first 1024-aligned shared address after the queues */
    const unsigned raw_sa = smem_addr(dense_smem_raw);
    const unsigned stage_sa =
        (raw_sa + (unsigned)dense_stage_offset<T>() + kStageAlign - 1) & ~(unsigned)(kStageAlign - 1);
    PackedStage &S = *reinterpret_cast<PackedStage *>(dense_smem_raw + (stage_sa - raw_sa));
    unsigned phases = 0u;      /* bit b: parity of buffer b's next TMA completion */
    unsigned pending = 0u;     /* bit b: a TMA copy into buffer b is outstanding   */
    bool failed = false;
    if constexpr (SRC == kSrcPacked && sizeof(T) == 4) {
        if (lane == 0) {
            mbar_init(smem_addr(&S.bar[wid][0]));
            mbar_init(smem_addr(&S.bar[wid][1]));
            asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        }
        __syncwarp();
    }
    /* wait for buffer b's TMA copy, at most kWaitLimit rounds; a wait that gives up
     * marks the status and stops the warp's work */
    auto wait_buf = [&](int b) {
        if (!((pending >> b) & 1u)) return;
        bool ok = false;
        const unsigned bar = smem_addr(&S.bar[wid][0]) + 8u * (unsigned)b;
        for (long long i = 0; i < kWaitLimit && !ok; i++)
            ok = mbar_try_wait(bar, (phases >> b) & 1u);
        ok = __all_sync(0xffffffffu, ok);
        if (!ok) {
            if (lane == 0 && a.err) atomicOr(a.err, 1 << CBC_ERR_CUDA);
            failed = true;
        }
        phases ^= 1u << b;
        pending &= ~(1u << b);
    };
    const bool grad = K != CBC_RECTANGULAR && !(a.st && (a.st->flags & kFatal));
    SlotPair<T> sp;
    sp.A.id = sp.B.id = -1;
    sp.mru_a = false;
    #pragma unroll
    for (int k = 0; k < 5; k++) sp.A.s[k] = sp.B.s[k] = T(0);
    T loss = T(0);
    const long long n_tasks = (a.n_items + 31) / 32;
    #pragma unroll 1
    while (true) {
        long long task = 0;
        if (lane == 0) task = (long long)atomicAdd(a.tasks, 1ull);
        task = __shfl_sync(0xffffffffu, task, 0);
        if (task >= n_tasks || failed) break;
        const long long it = task * 32 + lane;
        long long c = a.n_chunks;
        int x = 0, y = 0;
        if (it < a.n_items) {
            const long long band = it / a.pitch;
            c = band * kPatchRows * a.pitch + (it - band * a.pitch);
            if (c < a.n_chunks) {
                const long long rem = (c * kChunk) % ((long long)a.H * a.W);
                y = (int)(rem / a.W);
                x = (int)(rem - (long long)y * a.W);
            }
        }
        if constexpr (SRC == kSrcPacked && sizeof(T) == 4)
            if (stage_row(S.pk[wid][0], S.tg[wid][0], smem_addr(&S.bar[wid][0]), lane, c, a,
                          &tm_pk, &tm_tg))
                pending |= 1u;
        /* every lane of the warp takes part in each chunk row (the queue is shared) */
        #pragma unroll 1
        for (int k = 0; k < kPatchRows; k++, c += a.pitch) {
            const bool live = c < a.n_chunks;
            const long long p0 = c * kChunk;
            if (k > 0 && live) advance_px(x, y, (a.pitch - 1) * kChunk, a.W, a.H);
            unsigned drawn = 0;
            int ln[kChunk];
            T gv[kChunk];
            #pragma unroll
            for (int e = 0; e < kChunk; e++) {
                ln[e] = -1;
                gv[e] = T(0);
            }
            if constexpr (SRC == kSrcPacked && sizeof(T) == 4) {
                const int buf = k & 1;
                /* the next chunk row's copy goes out before this row is read */
                if (k + 1 < kPatchRows &&
                    stage_row(S.pk[wid][buf ^ 1], S.tg[wid][buf ^ 1],
                              smem_addr(&S.bar[wid][buf ^ 1]), lane, c + a.pitch, a, &tm_pk,
                              &tm_tg))
                    pending |= 1u << (buf ^ 1);
                wait_buf(buf);
                if (failed) break;
                __syncwarp();                /* the lanes' own stores of a loaded row */
                if (live) {
                    unsigned long long wv[kChunk];
                    float tv[kChunk];
                    uint4 q[kPkPieces], r[kTgPieces];
                    const unsigned bp = smem_addr(S.pk[wid][buf]), bt = smem_addr(S.tg[wid][buf]);
                    #pragma unroll
                    for (int j = 0; j < kPkPieces; j++)
                        q[j] = *reinterpret_cast<const uint4 *>(S.pk[wid][buf] + swz<64>(bp, lane, j));
                    #pragma unroll
                    for (int j = 0; j < kTgPieces; j++)
                        r[j] = *reinterpret_cast<const uint4 *>(S.tg[wid][buf] + swz<32>(bt, lane, j));
                    __builtin_memcpy(wv, q, sizeof(wv));
                    __builtin_memcpy(tv, r, sizeof(tv));
                    unsigned nz = 0;
                    #pragma unroll
                    for (int e = 0; e < kChunk; e++) {
                        nz |= (wv[e] != 0ull ? 1u : 0u) << e;
                        ln[e] = (int)(0xffffffffu - (unsigned)wv[e]);
                        drawn |= (wv[e] != 0ull && (unsigned)ln[e] < (unsigned)a.n_lines ? 1u : 0u)
                                 << e;
                        const T v = (T)__uint_as_float((unsigned)(wv[e] >> 32));
                        if (wv[e] != 0ull) loss += v * (v - T(2) * (T)tv[e]);
                        gv[e] = T(2) * (v - (T)tv[e]);
                    }
                    if (nz && a.clear) {
                        if (a.vec && p0 + kChunk <= a.n_px) {
                            uint4 *dst = reinterpret_cast<uint4 *>(a.clear + p0);
                            #pragma unroll
                            for (int i = 0; i < kChunk / 2; i++) dst[i] = make_uint4(0, 0, 0, 0);
                        } else {
                            #pragma unroll
                            for (int e = 0; e < kChunk; e++)
                                if (wv[e]) a.clear[p0 + e] = 0ull;
                        }
                    }
                }
            } else if (live) {
                load_chunk(a.winner, p0, a.n_px, a.vec, ln);
                #pragma unroll
                for (int e = 0; e < kChunk; e++)
                    drawn |= ((unsigned)ln[e] < (unsigned)a.n_lines ? 1u : 0u) << e;
                if (drawn && grad) {
                    if (a.grad_out) {
                        load_chunk(a.grad_out, p0, a.n_px, a.vec, gv);
                    } else {
                        T iv[kChunk], tv[kChunk];
                        load_chunk(a.image, p0, a.n_px, a.vec, iv);
                        load_chunk(a.target, p0, a.n_px, a.vec, tv);
                        #pragma unroll
                        for (int e = 0; e < kChunk; e++) gv[e] = T(2) * (iv[e] - tv[e]);
                    }
                }
            }
            /* the pixels with a term, compacted into the warp's queue in pixel order */
            unsigned work = 0;
            if (grad) {
                #pragma unroll
                for (int e = 0; e < kChunk; e++)
                    work |= (((drawn >> e) & 1u) && gv[e] != T(0) ? 1u : 0u) << e;
            }
            const int cnt = __popc(work);
            int incl = cnt;
            #pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            if (total > 0) {
                const int off = incl - cnt;
                Q.x[wid][lane] = x;
                Q.y[wid][lane] = y;
                #pragma unroll
                for (int e = 0; e < kChunk; e++) {
                    if ((work >> e) & 1u) {
                        const int q = qslot(off + __popc(work & ((1u << e) - 1u)));
                        Q.line[wid][q] = ln[e];
                        Q.g[wid][q] = gv[e];
                        Q.pos[wid][q] = (unsigned char)((lane << 3) | e);
                    }
                }
                __syncwarp();
                /* lane l takes the contiguous entries [l m, l m + m): neighbouring
                 * pixels, mostly of one or two lines */
                const int m = (total + 31) >> 5;
                #pragma unroll 1
                for (int r = 0; r < m; r++) {
                    const int i = lane * m + r;
                    if (i < total) {
                        const int q = qslot(i);
                        const int line = Q.line[wid][q];
                        const T g = Q.g[wid][q];
                        const int pos = Q.pos[wid][q];
                        int xe = Q.x[wid][pos >> 3], ye = Q.y[wid][pos >> 3];
                        advance_px(xe, ye, pos & 7, a.W, a.H);
                        sp.template add<K>(a, line, g, (T)xe, (T)ye);
                    }
                }
                __syncwarp();
            }
            if (live) advance_px(x, y, kChunk, a.W, a.H);
        }
    }
    /* a warp that stopped on a failed wait still waits (bounded) for its other copy */
    if constexpr (SRC == kSrcPacked && sizeof(T) == 4) {
        wait_buf(0);
        wait_buf(1);
    }
    sp.A.flush(a.gacc);
    sp.B.flush(a.gacc);
    if (SRC == kSrcPacked && a.partials) {
        __shared__ double red[kDenseWarps];
        double l = (double)loss;
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
        if (lane == 0) red[wid] = l;
        __syncthreads();
        if (threadIdx.x == 0) {
            double b = 0.0;
            for (int w = 0; w < kDenseWarps; w++) b += red[w];
            a.partials[blockIdx.x] = b;
        }
    }
}

template <typename T>
struct AdjArgs {
    DriveArgs<T> d;
    const T *lines;
    const T *grad_out;
    const T *image;
    const T *out0;
    const T *target;
    int *winner;
    double *gacc;
    T max_val;
};

template <typename T, int K>
__global__ void __launch_bounds__(kSegWarps * 32)
winner_kernel(AdjArgs<T> a)
{
    WinnerAct<T, K> act;
    act.image = a.image;
    act.out0 = a.out0;
    act.winner = a.winner;
    act.max_val = a.max_val;
    act.W = a.d.W;
    act.gtab = stage_gauss_table<T, K>();
    drive_segments(a.d, act);
}

template <typename T, int K>
__global__ void __launch_bounds__(kSegWarps * 32)
backward_kernel(AdjArgs<T> a)
{
    __shared__ T acc_s[kSegWarps][32][5];
    __shared__ GradCoef<T> coef_s[kSegWarps][32];
    BackwardAct<T, K> act;
    act.lines = a.lines;
    act.grad_out = a.grad_out;
    act.image = a.image;
    act.target = a.target;
    act.gacc = a.gacc;
    act.acc = acc_s[threadIdx.x >> 5];
    act.coef = coef_s[threadIdx.x >> 5];
    act.max_val = a.max_val;
    act.W = a.d.W;
    drive_segments(a.d, act);
}

/* grad_lines = gacc in T; with partials, block 0 also sums the dense pass's per-block
 * loss partials into *loss */
template <typename T>
__global__ void __launch_bounds__(256)
finalize_kernel(const double *gacc, T *grad_lines, long long n, const double *partials,
                int n_partials, double *loss)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) grad_lines[i] = (T)gacc[i];
    if (loss && blockIdx.x == 0) {
        __shared__ double red[8];
        double v = 0.0;
        for (int k = threadIdx.x; k < n_partials; k += blockDim.x) v += partials[k];
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            double b = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) b += red[w];
            *loss = b;
        }
    }
}

struct AdjLayout {
    size_t status, recs, cks, gacc, coef, total;
};

AdjLayout adj_layout(long long n_lines, long long ck_capacity, size_t rec_bytes, size_t ck_bytes,
                     size_t coef_bytes)
{
    auto up = [](size_t v) { return (v + 255) / 256 * 256; };
    AdjLayout L;
    size_t off = 0;
    L.status = off; off = up(off + sizeof(DevStatus));
    L.recs = off;   off = up(off + rec_bytes * (size_t)n_lines);
    L.cks = off;    off = up(off + ck_bytes * (size_t)ck_capacity);
    L.gacc = off;   off = up(off + sizeof(double) * (5 * (size_t)n_lines + 1));
    L.coef = off;   off = up(off + coef_bytes * (size_t)n_lines);
    L.total = off;
    return L;
}

inline bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

/* thread items of a dense pass over n_px pixels of width W: patches of kPatchRows
 * chunks, pitch chunks per row step */
inline int dense_pitch(long long W)
{
    const long long p = (W + kChunk / 2) / kChunk;
    return (int)(p < 1 ? 1 : p);
}

inline long long dense_items(long long n_px, long long W)
{
    const long long chunks = (n_px + kChunk - 1) / kChunk;
    const long long band = (long long)kPatchRows * dense_pitch(W);
    return (chunks + band - 1) / band * dense_pitch(W);
}

/* fills the sizes, pitch and alignment of a dense pass over n_frames x H x W pixels */
template <typename T>
void dense_shape(DenseArgs<T> &a, long long n_frames, long long H, long long W)
{
    a.H = (int)H;
    a.W = (int)W;
    a.n_px = n_frames * H * W;
    a.n_chunks = (a.n_px + kChunk - 1) / kChunk;
    a.n_full = a.n_px / kChunk;
    a.pitch = dense_pitch(W);
    a.n_items = dense_items(a.n_px, W);
    a.vec = aligned16(a.packed) && aligned16(a.clear) && aligned16(a.winner) &&
            aligned16(a.grad_out) && aligned16(a.image) && aligned16(a.target);
}

/* cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link) */
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled()
{
    static std::atomic<void *> fp{nullptr};
    static std::atomic<int> tried{0};
    void *p = fp.load(std::memory_order_acquire);
    if (!p && !tried.load(std::memory_order_acquire)) {
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        fp.store(p, std::memory_order_release);
        tried.store(1, std::memory_order_release);
    }
    return reinterpret_cast<EncodeTiledFn>(p);
}

/* the tensor maps of the packed pass: the packed words and the targets as 2-D arrays
 * of whole chunks (kChunk elements x n_full chunks), boxes of 32 chunks, swizzled 64 B
 * and 32 B; false when they cannot be made (the pass then loads every row itself) */
template <typename T>
bool encode_packed_maps(const DenseArgs<T> &a, CUtensorMap *pk, CUtensorMap *tg)
{
    if (a.n_full < 32 || a.n_full > 0x7fffffffll || !a.packed || !a.target) return false;
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)kChunk, (cuuint64_t)a.n_full};
    const cuuint32_t box[2] = {(cuuint32_t)kChunk, 32u};
    const cuuint32_t estr[2] = {1u, 1u};
    const cuuint64_t spk[1] = {(cuuint64_t)kChunk * 8};
    const cuuint64_t stg[1] = {(cuuint64_t)kChunk * 4};
    if (enc(pk, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2,
            const_cast<unsigned long long *>(a.packed), dims, spk, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    if (enc(tg, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<T *>(a.target), dims, stg, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    return true;
}

/* the coefficient table of the lines, then the persistent pass: as many blocks as
 * fit on the GPU (at most kDenseMaxBlocks); *blocks = the grid (loss partials) */
template <typename T, int K, int SRC>
cudaError_t launch_dense_k(const DenseArgs<T> &a, const T *lines, T max_val, cudaStream_t s,
                           int *blocks)
{
    GradCoef<T> *coef = const_cast<GradCoef<T> *>(a.coef);
    if (a.n_lines > 0) {
        grad_coef_kernel<T, K><<<(unsigned)((a.n_lines + 255) / 256), 256, 0, s>>>(
            lines, a.n_lines, max_val, coef);
        note_launches(1);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (blocks) *blocks = 0;
    if (a.n_items < 1) return cudaSuccess;
    CUtensorMap tm_pk, tm_tg;
    DenseArgs<T> args = a;
    args.tma = 0;
    if constexpr (SRC == kSrcPacked && sizeof(T) == 4)
        args.tma = args.vec && encode_packed_maps(a, &tm_pk, &tm_tg) ? 1 : 0;
    if (!args.tma) {
        memset(&tm_pk, 0, sizeof tm_pk);
        memset(&tm_tg, 0, sizeof tm_tg);
    }
    auto fn = dense_max_kernel<T, K, SRC>;
    constexpr size_t smem = dense_smem<T, SRC>();
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
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kDenseThreads, smem);
        g = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
        if (g > kDenseMaxBlocks) g = kDenseMaxBlocks;
        grid_cache[dev & 63].store(g, std::memory_order_relaxed);
    }
    const long long need = (a.n_items + kDenseThreads - 1) / kDenseThreads;
    const int grid = need < g ? (int)need : g;
    fn<<<grid, kDenseThreads, smem, s>>>(args, tm_pk, tm_tg);
    note_launches(1);
    if (blocks) *blocks = grid;
    return cudaGetLastError();
}

template <typename T, int SRC>
cudaError_t launch_dense(const DenseArgs<T> &a, const T *lines, T max_val, int kernel,
                         cudaStream_t s, int *blocks = nullptr)
{
    switch (kernel) {
    case CBC_BIWEIGHT:    return launch_dense_k<T, CBC_BIWEIGHT, SRC>(a, lines, max_val, s, blocks);
    case CBC_GAUSSIAN:    return launch_dense_k<T, CBC_GAUSSIAN, SRC>(a, lines, max_val, s, blocks);
    case CBC_PARABOLIC:   return launch_dense_k<T, CBC_PARABOLIC, SRC>(a, lines, max_val, s, blocks);
    case CBC_RECTANGULAR: return launch_dense_k<T, CBC_RECTANGULAR, SRC>(a, lines, max_val, s, blocks);
    default:              return launch_dense_k<T, CBC_TRIANGULAR, SRC>(a, lines, max_val, s, blocks);
    }
}

template <typename T, int K>
cudaError_t launch_walks(const AdjArgs<T> &aa, int overlap, cudaStream_t s)
{
    if (overlap == CBC_MAX) {
        const unsigned grid = resident_grid(winner_kernel<T, K>, kSegWarps * 32);
        winner_kernel<T, K><<<grid, kSegWarps * 32, 0, s>>>(aa);
    } else {
        backward_kernel<T, K><<<resident_grid(backward_kernel<T, K>, kSegWarps * 32),
                                kSegWarps * 32, 0, s>>>(aa);
    }
    note_launches(1);
    return cudaGetLastError();
}

template <typename T>
int backward_impl(const T *grad_out, long long n_frames, long long H, long long W,
                  const T *lines, long long n_lines, const void *idxs, int idx_bytes,
                  T max_val, int kernel, int overlap, const T *image, const T *out0,
                  int *winner, T *grad_lines, void *workspace, size_t ws_bytes,
                  long long ck_capacity, void *stream, const T *target = nullptr,
                  bool winner_known = false, const unsigned long long *packed = nullptr)
{
    if (packed) winner_known = true;
    clear_error();
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
    if (n_lines > INT_MAX) return fail(CBC_ERR_INVALID, "too many lines");
    if (ck_capacity < 0 || ck_capacity > INT_MAX)
        return fail(CBC_ERR_INVALID, "checkpoint_capacity out of range");
    const bool pixels = n_frames * H * W > 0;
    if (n_lines > 0 && (!lines || !grad_lines)) return fail(CBC_ERR_INVALID, "null pointer");
    if (n_lines > 0 && pixels && !grad_out && !(target && (image || packed)))
        return fail(CBC_ERR_INVALID, "null grad_out");
    if (overlap == CBC_MAX && n_lines > 0 && pixels && !packed && (!image || !winner))
        return fail(CBC_ERR_INVALID, "max overlap needs the forward image and a winner buffer");
    if (packed && (overlap != CBC_MAX || sizeof(T) != sizeof(float) || !target))
        return fail(CBC_ERR_INVALID, "packed winners are for the float32 max-overlap squared loss");
    AdjLayout L = adj_layout(n_lines, ck_capacity, sizeof(LineRec<T>), sizeof(Checkpoint<T>),
                             sizeof(GradCoef<T>));
    if (!workspace || ws_bytes < L.total)
        return fail(CBC_ERR_INVALID, "workspace too small (" + std::to_string(ws_bytes) + " < " +
                                         std::to_string(L.total) + ")");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    DevStatus *st = reinterpret_cast<DevStatus *>(ws + L.status);
    LineRec<T> *recs = reinterpret_cast<LineRec<T> *>(ws + L.recs);
    Checkpoint<T> *cks = reinterpret_cast<Checkpoint<T> *>(ws + L.cks);
    double *gacc = reinterpret_cast<double *>(ws + L.gacc);
    init_status_kernel<<<1, 1, 0, s>>>(st, CBC_STRATEGY_LINES);
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (n_lines == 0) return CBC_OK;
    /* the (N, 5) sums and, after them, the dense pass's task counter */
    e = cudaMemsetAsync(gacc, 0, sizeof(double) * (5 * (size_t)n_lines + 1), s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    /* the walks (sum overlap, and the winner pass of max overlap) need the line records
     * and walk checkpoints; the dense max pass needs only the lines */
    const bool walks = pixels && (overlap == CBC_SUM || !winner_known);
    if (walks) {
        Geometry g;
        g.H = (int)H;
        g.W = (int)W;
        g.tile_w = g.tile_h = 64;
        g.tiles_x = g.tiles_y = 1;
        const unsigned nb = (unsigned)((n_lines + 255) / 256);
        if (idxs && idx_bytes == 8)
            prep_kernel<T, int64_t, false, true><<<nb, 256, 0, s>>>(
                lines, idxs, n_lines, n_frames, g, recs, nullptr, cks, ck_capacity, st, nullptr);
        else
            prep_kernel<T, int32_t, false, true><<<nb, 256, 0, s>>>(
                lines, idxs, n_lines, n_frames, g, recs, nullptr, cks, ck_capacity, st, nullptr);
        note_launches(1);
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
        if (overlap == CBC_MAX) {
            e = cudaMemsetAsync(winner, 0x7f, sizeof(int) * (size_t)(n_frames * H * W), s);
            if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
        }
        AdjArgs<T> aa;
        aa.d.recs = recs;
        aa.d.cks = cks;
        aa.d.H = (int)H;
        aa.d.W = (int)W;
        aa.d.st = st;
        aa.d.work = &st->work;
        aa.lines = lines;
        aa.grad_out = grad_out;
        aa.image = image;
        aa.out0 = out0;
        aa.target = target;
        aa.winner = winner;
        aa.gacc = gacc;
        aa.max_val = max_val;
        switch (kernel) {
        case CBC_BIWEIGHT:    e = launch_walks<T, CBC_BIWEIGHT>(aa, overlap, s); break;
        case CBC_GAUSSIAN:    e = launch_walks<T, CBC_GAUSSIAN>(aa, overlap, s); break;
        case CBC_PARABOLIC:   e = launch_walks<T, CBC_PARABOLIC>(aa, overlap, s); break;
        case CBC_RECTANGULAR: e = launch_walks<T, CBC_RECTANGULAR>(aa, overlap, s); break;
        default:              e = launch_walks<T, CBC_TRIANGULAR>(aa, overlap, s); break;
        }
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    }
    if (pixels && overlap == CBC_MAX) {
        DenseArgs<T> da{};
        da.packed = packed;
        da.winner = winner;
        da.grad_out = grad_out;
        da.image = image;
        da.target = target;
        da.coef = reinterpret_cast<GradCoef<T> *>(ws + L.coef);
        da.gacc = gacc;
        da.tasks = reinterpret_cast<unsigned long long *>(gacc + 5 * n_lines);
        da.st = walks ? st : nullptr;
        da.err = &st->flags;
        da.n_lines = (int)n_lines;
        dense_shape(da, n_frames, H, W);
        if constexpr (sizeof(T) == 4) {
            e = packed ? launch_dense<T, kSrcPacked>(da, lines, max_val, kernel, s)
                       : launch_dense<T, kSrcWinner>(da, lines, max_val, kernel, s);
        } else {
            e = launch_dense<T, kSrcWinner>(da, lines, max_val, kernel, s);
        }
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    }
    const long long n5 = 5 * n_lines;
    finalize_kernel<T><<<(unsigned)((n5 + 255) / 256), 256, 0, s>>>(gacc, grad_lines, n5, nullptr,
                                                                    0, nullptr);
    note_launches(1);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    return CBC_OK;
}

/* the step workspace: the forward's (lines strategy) followed by the (N, 5) sums, the
 * lines' coefficient table and the dense pass's per-block loss partials */
struct StepLayout {
    size_t draw, gacc, coef, partials, total;
};

bool step_layout(long long n_frames, long long H, long long W, long long n_lines,
                 long long capacity, long long ck_capacity, StepLayout &L)
{
    auto up = [](size_t v) { return (v + 255) / 256 * 256; };
    cbc_tuning t{};
    t.strategy = CBC_STRATEGY_LINES;
    L.draw = cbc_draw_lines_workspace_size(n_frames, H, W, n_lines, capacity, ck_capacity, 4, &t);
    if (L.draw == 0) return false;
    size_t off = up(L.draw);
    L.gacc = off;     off = up(off + sizeof(double) * (5 * (size_t)n_lines + 1));
    L.coef = off;     off = up(off + sizeof(GradCoef<float>) * (size_t)n_lines);
    L.partials = off; off = up(off + sizeof(double) * kDenseMaxBlocks);
    L.total = off;
    return true;
}

int loss_step_impl(const float *target, long long n_frames, long long H, long long W,
                   const float *lines, long long n_lines, const void *idxs, int idx_bytes,
                   float max_val, int kernel, unsigned long long *packed, float *grad_lines,
                   double *loss, void *workspace, size_t ws_bytes, long long capacity,
                   long long ck_capacity, void *stream)
{
    clear_error();
    if (n_frames < 0 || H < 0 || W < 0 || n_lines < 0 || capacity < 0 || ck_capacity < 0)
        return fail(CBC_ERR_INVALID, "negative size");
    const bool pixels = n_frames * H * W > 0;
    if (n_lines > 0 && (!lines || !grad_lines)) return fail(CBC_ERR_INVALID, "null pointer");
    if (pixels && (!target || !packed)) return fail(CBC_ERR_INVALID, "null target or packed");
    StepLayout L;
    if (!step_layout(n_frames, H, W, n_lines, capacity, ck_capacity, L))
        return fail(CBC_ERR_INVALID, "invalid sizes");
    if (!workspace || ws_bytes < L.total)
        return fail(CBC_ERR_INVALID, "workspace too small (" + std::to_string(ws_bytes) + " < " +
                                         std::to_string(L.total) + ")");
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    /* the forward: value and winner packed per pixel, no frames written */
    int rc = cbc_draw_lines_max_winner_f32(nullptr, nullptr, reinterpret_cast<uint64_t *>(packed),
                                           n_frames, H, W, lines, n_lines, idxs, idx_bytes,
                                           max_val, kernel, workspace, L.draw, capacity,
                                           ck_capacity, stream);
    if (rc != CBC_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double *gacc = reinterpret_cast<double *>(ws + L.gacc);
    double *partials = reinterpret_cast<double *>(ws + L.partials);
    cudaError_t e = cudaSuccess;
    e = cudaMemsetAsync(gacc, 0, sizeof(double) * (5 * (size_t)n_lines + 1), s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    int blocks = 0;
    if (pixels) {
        DenseArgs<float> da{};
        da.packed = packed;
        da.clear = packed;
        da.target = target;
        da.coef = reinterpret_cast<GradCoef<float> *>(ws + L.coef);
        da.gacc = gacc;
        da.tasks = reinterpret_cast<unsigned long long *>(gacc + 5 * n_lines);
        da.partials = loss ? partials : nullptr;
        da.st = reinterpret_cast<const DevStatus *>(ws);   /* the forward's status block */
        da.err = &reinterpret_cast<DevStatus *>(ws)->flags;
        da.n_lines = (int)n_lines;
        dense_shape(da, n_frames, H, W);
        e = launch_dense<float, kSrcPacked>(da, lines, max_val, kernel, s, &blocks);
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    }
    const long long n5 = 5 * n_lines;
    if (n5 > 0 || loss) {
        const long long nb = n5 > 0 ? (n5 + 255) / 256 : 1;
        finalize_kernel<float><<<(unsigned)nb, 256, 0, s>>>(gacc, grad_lines, n5, partials,
                                                             blocks, loss);
        note_launches(1);
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    }
    return CBC_OK;
}

/* sum over the frames of (image - target)^2 into *loss (zeroed before) */
__global__ void __launch_bounds__(256)
sq_diff_kernel(const float *__restrict__ image, const float *__restrict__ target, long long n,
               double *loss)
{
    __shared__ double warp_sums[8];
    double acc = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double d = (double)image[i] - (double)target[i];
        acc += d * d;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < 8; w++) b += warp_sums[w];
        atomicAdd(loss, b);
    }
}

/* the sum-overlap squared-loss step: the forward into `image` (zeroed first) with the
 * lines strategy, then the adjoint walks over the forward's own line records and walk
 * checkpoints (no second prep), then the (N, 5) gradient and, if asked, the loss */
int sum_loss_step_impl(const float *target, float *image, long long n_frames, long long H,
                       long long W, const float *lines, long long n_lines, const void *idxs,
                       int idx_bytes, float max_val, int kernel, float *grad_lines,
                       double *loss, void *workspace, size_t ws_bytes, long long capacity,
                       long long ck_capacity, void *stream)
{
    clear_error();
    if (n_frames < 0 || H < 0 || W < 0 || n_lines < 0 || capacity < 0 || ck_capacity < 0)
        return fail(CBC_ERR_INVALID, "negative size");
    const long long px = n_frames * H * W;
    if (n_lines > 0 && (!lines || !grad_lines)) return fail(CBC_ERR_INVALID, "null pointer");
    if (px > 0 && (!target || !image)) return fail(CBC_ERR_INVALID, "null target or image");
    StepLayout L;
    if (!step_layout(n_frames, H, W, n_lines, capacity, ck_capacity, L))
        return fail(CBC_ERR_INVALID, "invalid sizes");
    if (!workspace || ws_bytes < L.total)
        return fail(CBC_ERR_INVALID, "workspace too small (" + std::to_string(ws_bytes) + " < " +
                                         std::to_string(L.total) + ")");
    cbc_tuning t{};
    t.strategy = CBC_STRATEGY_LINES;
    size_t recs_off = 0, cks_off = 0;
    if (!draw_workspace_parts(n_frames, H, W, n_lines, capacity, ck_capacity, 4, &t, &recs_off,
                              &cks_off))
        return fail(CBC_ERR_INVALID, "invalid sizes");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaSuccess;
    if (px > 0) e = cudaMemsetAsync(image, 0, sizeof(float) * (size_t)px, s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    int rc = cbc_draw_lines_f32(image, n_frames, H, W, lines, n_lines, idxs, idx_bytes, max_val,
                                kernel, CBC_SUM, workspace, L.draw, capacity, ck_capacity, &t,
                                stream);
    if (rc != CBC_OK) return rc;
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    DevStatus *st = reinterpret_cast<DevStatus *>(ws);      /* the forward's status block */
    double *gacc = reinterpret_cast<double *>(ws + L.gacc);
    e = cudaMemsetAsync(gacc, 0, sizeof(double) * (5 * (size_t)n_lines + 1), s);
    /* the forward's render consumed the work counter; the adjoint walks start it again */
    if (e == cudaSuccess) e = cudaMemsetAsync(&st->work, 0, sizeof(st->work), s);
    if (e == cudaSuccess && loss) e = cudaMemsetAsync(loss, 0, sizeof(double), s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (n_lines > 0 && px > 0) {
        AdjArgs<float> aa{};
        aa.d.recs = reinterpret_cast<const LineRec<float> *>(ws + recs_off);
        aa.d.cks = reinterpret_cast<const Checkpoint<float> *>(ws + cks_off);
        aa.d.H = (int)H;
        aa.d.W = (int)W;
        aa.d.st = st;
        aa.d.work = &st->work;
        aa.lines = lines;
        aa.image = image;
        aa.target = target;
        aa.gacc = gacc;
        aa.max_val = max_val;
        switch (kernel) {
        case CBC_BIWEIGHT:    e = launch_walks<float, CBC_BIWEIGHT>(aa, CBC_SUM, s); break;
        case CBC_GAUSSIAN:    e = launch_walks<float, CBC_GAUSSIAN>(aa, CBC_SUM, s); break;
        case CBC_PARABOLIC:   e = launch_walks<float, CBC_PARABOLIC>(aa, CBC_SUM, s); break;
        case CBC_RECTANGULAR: e = launch_walks<float, CBC_RECTANGULAR>(aa, CBC_SUM, s); break;
        default:              e = launch_walks<float, CBC_TRIANGULAR>(aa, CBC_SUM, s); break;
        }
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    }
    const long long n5 = 5 * n_lines;
    if (n5 > 0) {
        finalize_kernel<float><<<(unsigned)((n5 + 255) / 256), 256, 0, s>>>(
            gacc, grad_lines, n5, nullptr, 0, nullptr);
        note_launches(1);
    }
    if (loss && px > 0) {
        long long blocks = (px + 255) / 256;
        if (blocks > 4096) blocks = 4096;
        sq_diff_kernel<<<(unsigned)blocks, 256, 0, s>>>(image, target, px, loss);
        note_launches(1);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    return CBC_OK;
}

/* one Adam step on the (N, 5) line parameters with the width clamp:
 * m = m + (1 - b1)(g - m), v = b2 v + (1 - b2) g^2,
 * p -= (lr / (1 - b1^t)) m / (sqrt(v) / sqrt(1 - b2^t) + eps), widths >= min_width */
__global__ void __launch_bounds__(256)
adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
            float *__restrict__ v, long long n, float step_size, float bc2_sqrt, float b1,
            float b2, float eps, float min_width)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = m[i] + (1.0f - b1) * (gi - m[i]);
    const float vi = v[i] * b2 + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float pi = p[i] - step_size * (mi / (sqrtf(vi) / bc2_sqrt + eps));
    if (i % 5 == 4 && pi < min_width) pi = min_width;
    p[i] = pi;
}

}  // namespace cbc

extern "C" {

int cbc_squared_loss_step_sum_f32(const float *target, float *image, int64_t n_frames,
                                  int64_t height, int64_t width, const float *lines,
                                  int64_t n_lines, const void *idxs, int32_t idx_bytes,
                                  float max_val, int32_t kernel, float *grad_lines,
                                  double *loss, void *workspace, size_t workspace_bytes,
                                  int64_t pair_capacity, int64_t checkpoint_capacity,
                                  void *stream)
{
    return cbc::sum_loss_step_impl(target, image, n_frames, height, width, lines, n_lines, idxs,
                                   idx_bytes, max_val, kernel, grad_lines, loss, workspace,
                                   workspace_bytes, pair_capacity, checkpoint_capacity, stream);
}

int cbc_adam_step_f32(float *params, const float *grad, float *exp_avg, float *exp_avg_sq,
                      int64_t n_lines, int64_t step, float lr, float beta1, float beta2,
                      float eps, float min_width, void *stream)
{
    cbc::clear_error();
    if (n_lines < 0 || step < 1) return cbc::fail(CBC_ERR_INVALID, "n_lines < 0 or step < 1");
    if (!(beta1 >= 0.0f && beta1 < 1.0f && beta2 >= 0.0f && beta2 < 1.0f))
        return cbc::fail(CBC_ERR_INVALID, "betas must lie in [0, 1)");
    if (n_lines == 0) return CBC_OK;
    if (!params || !grad || !exp_avg || !exp_avg_sq) return cbc::fail(CBC_ERR_INVALID, "null pointer");
    const double bc1 = 1.0 - std::pow((double)beta1, (double)step);
    const double bc2 = 1.0 - std::pow((double)beta2, (double)step);
    const long long n = 5 * n_lines;
    cbc::adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        params, grad, exp_avg, exp_avg_sq, n, (float)(lr / bc1), (float)std::sqrt(bc2), beta1,
        beta2, eps, min_width);
    cbc::note_launches(1);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cbc::fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    return CBC_OK;
}


size_t cbc_draw_lines_backward_workspace_size(int64_t n_lines, int64_t checkpoint_capacity,
                                              int32_t elem_bytes)
{
    if (n_lines < 0 || checkpoint_capacity < 0) return 0;
    size_t rec = elem_bytes == 8 ? sizeof(cbc::LineRec<double>) : sizeof(cbc::LineRec<float>);
    size_t ck = elem_bytes == 8 ? sizeof(cbc::Checkpoint<double>) : sizeof(cbc::Checkpoint<float>);
    size_t coef = elem_bytes == 8 ? sizeof(cbc::GradCoef<double>) : sizeof(cbc::GradCoef<float>);
    return cbc::adj_layout(n_lines, checkpoint_capacity, rec, ck, coef).total;
}

int cbc_draw_lines_backward_f32(const float *grad_out, int64_t n_frames, int64_t height,
                                int64_t width, const float *lines, int64_t n_lines,
                                const void *idxs, int32_t idx_bytes, float max_val,
                                int32_t kernel, int32_t overlap, const float *image,
                                const float *out0, int32_t *winner, float *grad_lines,
                                void *workspace, size_t workspace_bytes,
                                int64_t checkpoint_capacity, void *stream)
{
    return cbc::backward_impl<float>(grad_out, n_frames, height, width, lines, n_lines, idxs,
                                     idx_bytes, max_val, kernel, overlap, image, out0, winner,
                                     grad_lines, workspace, workspace_bytes, checkpoint_capacity,
                                     stream);
}

int cbc_draw_lines_backward_f64(const double *grad_out, int64_t n_frames, int64_t height,
                                int64_t width, const double *lines, int64_t n_lines,
                                const void *idxs, int32_t idx_bytes, double max_val,
                                int32_t kernel, int32_t overlap, const double *image,
                                const double *out0, int32_t *winner, double *grad_lines,
                                void *workspace, size_t workspace_bytes,
                                int64_t checkpoint_capacity, void *stream)
{
    return cbc::backward_impl<double>(grad_out, n_frames, height, width, lines, n_lines, idxs,
                                      idx_bytes, max_val, kernel, overlap, image, out0, winner,
                                      grad_lines, workspace, workspace_bytes,
                                      checkpoint_capacity, stream);
}

int cbc_squared_loss_backward_f32(const float *image, const float *target, int64_t n_frames,
                                  int64_t height, int64_t width, const float *lines,
                                  int64_t n_lines, const void *idxs, int32_t idx_bytes,
                                  float max_val, int32_t kernel, int32_t overlap,
                                  const float *out0, int32_t *winner, float *grad_lines,
                                  void *workspace, size_t workspace_bytes,
                                  int64_t checkpoint_capacity, void *stream)
{
    if (!image || !target) return cbc::fail(CBC_ERR_INVALID, "null image or target");
    return cbc::backward_impl<float>(nullptr, n_frames, height, width, lines, n_lines, idxs,
                                     idx_bytes, max_val, kernel, overlap, image, out0, winner,
                                     grad_lines, workspace, workspace_bytes, checkpoint_capacity,
                                     stream, target);
}

int cbc_squared_loss_backward_f64(const double *image, const double *target, int64_t n_frames,
                                  int64_t height, int64_t width, const double *lines,
                                  int64_t n_lines, const void *idxs, int32_t idx_bytes,
                                  double max_val, int32_t kernel, int32_t overlap,
                                  const double *out0, int32_t *winner, double *grad_lines,
                                  void *workspace, size_t workspace_bytes,
                                  int64_t checkpoint_capacity, void *stream)
{
    if (!image || !target) return cbc::fail(CBC_ERR_INVALID, "null image or target");
    return cbc::backward_impl<double>(nullptr, n_frames, height, width, lines, n_lines, idxs,
                                      idx_bytes, max_val, kernel, overlap, image, out0, winner,
                                      grad_lines, workspace, workspace_bytes,
                                      checkpoint_capacity, stream, target);
}

int cbc_draw_lines_backward_ex_f32(const float *grad_out, const float *target, int64_t n_frames,
                                   int64_t height, int64_t width, const float *lines,
                                   int64_t n_lines, const void *idxs, int32_t idx_bytes,
                                   float max_val, int32_t kernel, int32_t overlap,
                                   const float *image, const float *out0, int32_t *winner,
                                   int32_t winner_known, const uint64_t *packed,
                                   float *grad_lines, void *workspace, size_t workspace_bytes,
                                   int64_t checkpoint_capacity, void *stream)
{
    if (!grad_out && !((image || packed) && target))
        return cbc::fail(CBC_ERR_INVALID, "null grad_out");
    return cbc::backward_impl<float>(grad_out, n_frames, height, width, lines, n_lines, idxs,
                                     idx_bytes, max_val, kernel, overlap, image, out0, winner,
                                     grad_lines, workspace, workspace_bytes, checkpoint_capacity,
                                     stream, grad_out ? nullptr : target, winner_known != 0,
                                     reinterpret_cast<const unsigned long long *>(packed));
}

int cbc_draw_lines_backward_ex_f64(const double *grad_out, const double *target, int64_t n_frames,
                                   int64_t height, int64_t width, const double *lines,
                                   int64_t n_lines, const void *idxs, int32_t idx_bytes,
                                   double max_val, int32_t kernel, int32_t overlap,
                                   const double *image, const double *out0, int32_t *winner,
                                   int32_t winner_known, const uint64_t *packed,
                                   double *grad_lines, void *workspace, size_t workspace_bytes,
                                   int64_t checkpoint_capacity, void *stream)
{
    if (packed) return cbc::fail(CBC_ERR_INVALID, "packed winners are for float32 max overlap");
    if (!grad_out && !(image && target)) return cbc::fail(CBC_ERR_INVALID, "null grad_out");
    return cbc::backward_impl<double>(grad_out, n_frames, height, width, lines, n_lines, idxs,
                                      idx_bytes, max_val, kernel, overlap, image, out0, winner,
                                      grad_lines, workspace, workspace_bytes,
                                      checkpoint_capacity, stream, grad_out ? nullptr : target,
                                      winner_known != 0);
}

size_t cbc_squared_loss_step_workspace_size(int64_t n_frames, int64_t height, int64_t width,
                                            int64_t n_lines, int64_t pair_capacity,
                                            int64_t checkpoint_capacity)
{
    if (n_frames < 0 || height < 0 || width < 0 || n_lines < 0 || pair_capacity < 0 ||
        checkpoint_capacity < 0)
        return 0;
    cbc::StepLayout L;
    if (!cbc::step_layout(n_frames, height, width, n_lines, pair_capacity, checkpoint_capacity, L))
        return 0;
    return L.total;
}

int cbc_squared_loss_step_f32(const float *target, int64_t n_frames, int64_t height,
                              int64_t width, const float *lines, int64_t n_lines,
                              const void *idxs, int32_t idx_bytes, float max_val, int32_t kernel,
                              uint64_t *packed, float *grad_lines, double *loss_delta,
                              void *workspace, size_t workspace_bytes, int64_t pair_capacity,
                              int64_t checkpoint_capacity, void *stream)
{
    return cbc::loss_step_impl(target, n_frames, height, width, lines, n_lines, idxs, idx_bytes,
                               max_val, kernel, reinterpret_cast<unsigned long long *>(packed),
                               grad_lines, loss_delta, workspace, workspace_bytes, pair_capacity,
                               checkpoint_capacity, stream);
}

}  // extern "C"
