/*
 * cbc_accumulate.cu — accumulate_lines for 2-D lines on sm_103a.
 *
 * Reference: accumulate_lines_nd_impl (cbclib_v2/_src/src/bresenham.cpp:151-259) and
 * its GPU counterpart (cuda_draw_lines.cu:467-523, :687-767, :948-1057).  Lines carry a
 * term index, terms a frame index.  Every term is drawn into a zeroed buffer of its own,
 * combining its lines with `in_overlap` (sum or std::max), and the pixels the term's
 * walks drew are then merged into out[frame(term)] with `out_overlap`.
 *
 * The pixels and their values are the forward's (drive_segments, cbc_common.cuh, over
 * walk checkpoints from prep_kernel).  The four overlap pairs map to:
 *   sum, sum  one L2 reduction per pixel: out += v (only the addition order differs
 *             from the reference's term-by-term sums);
 *   max, max  out = std::max(out, max(+0, v)): a term buffer starts at zero, so every
 *             pixel a term draws is merged with at least +0 (bit-exact);
 *   max, sum  a term's value at a pixel must be complete before it is merged.  Each
 *   sum, max  term is built in shared memory by one CTA (term_render2_kernel: an
 *             open-addressing (pixel, value) table, the term's columns shared out
 *             among the threads), then every drawn pixel is merged into out with one
 *             atomic.  A term with more pixels than the table holds is taken in
 *             partitions of its pixels, each pass keeping one partition.  Terms that
 *             would need more than kTerm2MaxParts partitions go instead through a
 *             (term, pixel) hash table in the workspace (key term << 32 | pixel, linear
 *             probing, at most 64 probes), combined there with atomics and merged by a
 *             pass over the table; when the workspace table is too small for them the
 *             call sets CBC_ERR_CAPACITY, draws nothing and pairs_needed names the
 *             capacity to retry with.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <limits.h>
#include <string>

#include "cbc_accumulate.cuh"

namespace cbc {

template <typename T, int K, int MODE>
struct AccumAct {
    static constexpr bool kNeedsError = true;
    T *out;
    T max_val;
    int W;
    const float *gtab;
    const int *term_of_line;
    unsigned long long *keys;
    T *vals;
    unsigned long long mask;       /* table capacity - 1 (a power of two) */
    const int *tbig;               /* per term: through the workspace table (mixed modes) */
    DevStatus *st;
    struct Pre {};
    /* with mixed overlaps this pass draws only the terms too large for shared memory */
    __device__ __forceinline__ bool keep_line(int line) const {
        if constexpr (MODE == kAccMaxSum || MODE == kAccSumMax) return tbig[term_of_line[line]] != 0;
        else return true;
    }
    template <class ST>
    __device__ __forceinline__ void item_begin(int, const ST &) {}
    __device__ __forceinline__ void item_end(int, const SlotTable<T> &) {}
    __device__ __forceinline__ Pre prefetch(const SlotTable<T> &, int, int, int) const { return {}; }
    __device__ __forceinline__ void pixel(const SlotTable<T> &S, int slot, int px, int py, T E,
                                          T, T, Pre) {
        using A = Ar<T>;
        const T v = A::mul(max_val, A::template profile_tab<K>(A::sqrt(E), gtab));
        const long long pix = (long long)py * W + px;
        if (MODE == kAccSumSum) {
            atomicAdd(out + S.fbase[slot] + pix, v);
        } else if (MODE == kAccMaxMax) {
            global_combine_max(out + S.fbase[slot] + pix, T(0) < v ? v : T(0));
        } else {
            table_combine<T, MODE & 1>(keys, vals, mask, term_of_line[S.line[slot]], pix, v, st);
        }
    }
};

template <typename T>
struct AccArgs {
    DriveArgs<T> d;
    T *out;
    T max_val;
    const int *term_of_line;
    unsigned long long *keys;
    T *vals;
    unsigned long long mask;
    const int *tbig;
    const int *nbig;               /* terms through the workspace table            */
    const float *big_est;          /* their estimated (term, pixel) pairs          */
    long long table_capacity;
};

template <typename T, int K, int MODE>
__global__ void __launch_bounds__(kSegWarps * 32, kSegMinBlocks)
accumulate_kernel(AccArgs<T> a)
{
    AccumAct<T, K, MODE> act;
    act.out = a.out;
    act.max_val = a.max_val;
    act.W = a.d.W;
    act.gtab = stage_gauss_table<T, K>();
    act.term_of_line = a.term_of_line;
    act.keys = a.keys;
    act.vals = a.vals;
    act.mask = a.mask;
    act.tbig = a.tbig;
    act.st = a.d.st;
    if constexpr (MODE == kAccMaxSum || MODE == kAccSumMax) {
        /* only the large terms, into a table at most half full by their estimate */
        if (!table_terms_fit(a.nbig, a.big_est, a.table_capacity, a.d.st)) return;
    }
    drive_segments(a.d, act);
}

template <typename T, int K>
cudaError_t launch_accumulate(const AccArgs<T> &a, int mode, cudaStream_t s)
{
    const unsigned threads = kSegWarps * 32;
    switch (mode) {
    case kAccSumSum:
        accumulate_kernel<T, K, kAccSumSum><<<resident_grid(accumulate_kernel<T, K, kAccSumSum>,
                                                            threads), threads, 0, s>>>(a);
        break;
    case kAccMaxSum:
        accumulate_kernel<T, K, kAccMaxSum><<<resident_grid(accumulate_kernel<T, K, kAccMaxSum>,
                                                            threads), threads, 0, s>>>(a);
        break;
    case kAccSumMax:
        accumulate_kernel<T, K, kAccSumMax><<<resident_grid(accumulate_kernel<T, K, kAccSumMax>,
                                                            threads), threads, 0, s>>>(a);
        break;
    default:
        accumulate_kernel<T, K, kAccMaxMax><<<resident_grid(accumulate_kernel<T, K, kAccMaxMax>,
                                                            threads), threads, 0, s>>>(a);
        break;
    }
    note_launches(1);
    return cudaGetLastError();
}

/* ---- mixed overlaps: terms built in shared memory ---------------------------------- */
template <typename T> struct Term2Table { static constexpr int kBits = 12; };   /* 4096 slots */
constexpr int kTerm2Threads = 256;
constexpr int kTerm2Blocks = 3;         /* resident CTAs per SM the budgets target    */
constexpr int kTerm2Stack = 64;         /* pending partitions per term                */
constexpr int kTerm2MaxParts = 8;       /* larger terms use the workspace table       */
constexpr float kTerm2Fill = 0.6f;      /* planned fill of the table per partition    */
constexpr unsigned kNoPixel = 0xffffffffu;

/* values, keys (pixel index within the frame) and the claimed slots in claim order */
template <typename T>
constexpr size_t term2_smem()
{
    return (size_t)(1 << Term2Table<T>::kBits) *
           (sizeof(T) + sizeof(unsigned) + sizeof(unsigned short));
}

template <typename T>
struct Term2Args {
    const LineRec<T> *recs;
    const Checkpoint<T> *cks;
    DevStatus *st;
    T *out;
    T max_val;
    int H, W;
    const int *tcount, *toff, *tlines, *tbig, *frame_of_term;
    const float *test;
    long long n_terms;
};

/* after prep: each drawable line adds itself to its term's count and its pixel estimate
 * to the term's, columns x (2 w len / |tangent along the long axis| + 1) */
template <typename T>
__global__ void __launch_bounds__(kThreads)
term_count2_kernel(const LineRec<T> *__restrict__ recs, const int *__restrict__ term_of_line,
                   long long n_lines, int *__restrict__ tcount, float *__restrict__ test)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_lines) return;
    const LineRec<T> &r = recs[i];
    if (!(r.flags & kDrawable) || r.ncols <= 0) return;
    const int t = term_of_line[i];
    atomicAdd(&tcount[t], 1);
    const float tl = fabsf((float)((r.flags & kAxisY) ? r.t1 : r.t0));
    const float span = tl > 0.0f ? 2.0f * (float)r.w * (float)r.len / tl + 1.0f : 1.0f;
    atomicAdd(&test[t], (float)r.ncols * span);
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
term_fill2_kernel(const LineRec<T> *__restrict__ recs, const int *__restrict__ term_of_line,
                  long long n_lines, int *__restrict__ tfill, int *__restrict__ tlines)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_lines) return;
    const LineRec<T> &r = recs[i];
    if (!(r.flags & kDrawable) || r.ncols <= 0) return;
    tlines[atomicAdd(&tfill[term_of_line[i]], 1)] = (int)i;
}

/* one term partition's pixels into the CTA's table: claim a slot (recording it in the
 * claim list) or find the pixel's, then combine with in_overlap; `full` is raised at
 * 3/4 of the table, after which the pass is discarded and redone in two halves */
template <typename T, int IN_MAX>
struct TermTable2 {
    unsigned *key;
    T *val;
    unsigned short *claimed;
    int *count, *full;
    unsigned pmask, part;
    __device__ __forceinline__ void add(unsigned pix, T v) const {
        constexpr int kBits = Term2Table<T>::kBits, kSize = 1 << kBits;
        if ((part_hash(pix) & pmask) != part) return;
        if (*reinterpret_cast<volatile int *>(full)) return;
        unsigned h = (pix * 2654435761u) >> (32 - kBits);      /* Fibonacci hashing */
        for (int p = 0; p < kSize; p++) {
            unsigned cur = *reinterpret_cast<volatile unsigned *>(key + h);
            if (cur == kNoPixel) {
                cur = atomicCAS(key + h, kNoPixel, pix);
                if (cur == kNoPixel) {
                    const int n = atomicAdd(count, 1);           /* < kSize: distinct slots */
                    claimed[n] = (unsigned short)h;
                    if (n >= kSize * 3 / 4) *reinterpret_cast<volatile int *>(full) = 1;
                }
            }
            if (cur == kNoPixel || cur == pix) {
                if (IN_MAX) term_combine_max(val + h, v);
                else atomicAdd(val + h, v);
                return;
            }
            h = (h + 1) & (kSize - 1);
        }
        *reinterpret_cast<volatile int *>(full) = 1;
    }
};

/* one CTA per term at a time (grid-stride over the terms the table path does not
 * take); the term's columns are shared out among the threads, each walking from its
 * segment checkpoint to its column and drawing the column's centre and spans exactly
 * as drive_segments does, then the claimed slots are merged into out and reset */
template <typename T, int K, int IN_MAX, int OUT_MAX>
__global__ void __launch_bounds__(kTerm2Threads, kTerm2Blocks)
term_render2_kernel(Term2Args<T> a)
{
    using A = Ar<T>;
    constexpr int kSize = 1 << Term2Table<T>::kBits;
    extern __shared__ __align__(16) unsigned char term2_smem_raw[];
    T *s_val = reinterpret_cast<T *>(term2_smem_raw);
    unsigned *s_key = reinterpret_cast<unsigned *>(term2_smem_raw + sizeof(T) * kSize);
    unsigned short *s_claimed = reinterpret_cast<unsigned short *>(
        term2_smem_raw + (sizeof(T) + sizeof(unsigned)) * kSize);
    __shared__ int s_pre[kTerm2Threads + 1];
    __shared__ int s_line[kTerm2Threads];
    __shared__ int s_warp[kTerm2Threads / 32];
    __shared__ unsigned s_stack[kTerm2Stack];
    __shared__ int s_depth, s_count, s_full;
    const float *gtab = stage_gauss_table<T, K>();
    if (a.st->flags & kFatal) return;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int j = tid; j < kSize; j += kTerm2Threads) {
        s_key[j] = kNoPixel;
        s_val[j] = T(0);
    }
    if (tid == 0) {
        s_count = 0;
        s_full = 0;
    }
    __syncthreads();
    const long long frame_px = (long long)a.H * a.W;
    const int W = a.W, H = a.H;
    for (long long t = blockIdx.x; t < a.n_terms; t += gridDim.x) {
        const int n_t = a.tcount[t];
        if (n_t == 0 || a.tbig[t]) continue;
        if (tid == 0) {
            /* at most kTerm2MaxParts starting partitions; a split adds one entry */
            const float want = a.test[t] / (kTerm2Fill * (float)kSize);
            int lg = 0;
            while ((float)(1 << lg) < want && (1 << lg) < kTerm2MaxParts) lg++;
            s_depth = 0;
            for (int p = (1 << lg) - 1; p >= 0; p--) s_stack[s_depth++] = ((unsigned)p << 5) | lg;
        }
        __syncthreads();
        while (s_depth > 0) {
            const unsigned top = s_stack[s_depth - 1];
            const unsigned lg = top & 31u, part = top >> 5;
            const TermTable2<T, IN_MAX> table{s_key, s_val, s_claimed, &s_count, &s_full,
                                              (1u << lg) - 1u, part};
            for (int c0 = 0; c0 < n_t && !s_full; c0 += kTerm2Threads) {
                /* this chunk's lines and the prefix sum of their columns */
                const int nc = min(kTerm2Threads, n_t - c0);
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
                if (tid == kTerm2Threads - 1) s_pre[kTerm2Threads] = before + incl;
                __syncthreads();
                const int total = s_pre[nc];
                for (int j = tid; j < total && !*reinterpret_cast<volatile int *>(&s_full);
                     j += kTerm2Threads) {
                    int lo = 0, hi = nc - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (s_pre[mid] <= j) lo = mid;
                        else hi = mid - 1;
                    }
                    const int line = s_line[lo], col = j - s_pre[lo];
                    const LineRec<T> r = a.recs[line];
                    const Checkpoint<T> ck = a.cks[r.ck_base + col / kCkCols];
                    if (ck.cx == INT_MIN) continue;
                    /* the walk from the checkpoint to the column: the position whose
                     * next move steps the long axis at walk index col */
                    Walker<T> wk;
                    wk.init(r);
                    wk.cx = ck.cx;
                    wk.cy = ck.cy;
                    wk.te = ck.te;
                    wk.ne = ck.ne;
                    const int ax = r.flags & kAxisY;
                    const int sa = ax ? wk.sy : wk.sx;
                    bool found = false;
                    int c = 0, sc = 0;
                    T te_c = T(0), ne_c = T(0);
                    int guard = 0;
                    while (wk.cx != r.x1 && wk.cy != r.y1) {
                        const typename Walker<T>::Next mv = wk.decide();
                        const int cc = ax ? wk.cy : wk.cx;
                        const int idx = (cc - r.c0) * sa;
                        if (idx > col) break;
                        if (idx == col && (ax ? mv.ny : mv.nx)) {
                            found = true;
                            c = cc;
                            sc = ax ? wk.cx : wk.cy;
                            te_c = wk.te;
                            ne_c = wk.ne;
                            break;
                        }
                        wk.step(mv);
                        if (++guard > 4 * CBC_MAX_WALK + 64) {
                            atomicOr(&a.st->flags, 1 << CBC_ERR_RANGE);
                            break;
                        }
                    }
                    if (!found) continue;
                    SlotParams<T> p;
                    p.len = r.len;
                    p.rlen = r.rlen;
                    p.ww = r.ww;
                    p.rww = r.rww;
                    p.len2 = r.len2;
                    p.fast = (r.flags & kFastDiv) ? 1 : 0;
                    const T len2 = r.len2, thr = r.ne_thr;
                    const T ts = ax ? r.t0 : r.t1, ns = ax ? r.t1 : -r.t0;
                    const int s_hi = (ax ? W : H) - 1;
                    auto pixel = [&](T te, T ne, int s) {
                        const bool cap = te < T(0) || te > len2;
                        const T nf = A::nterm(ne, p);
                        const T E = cap ? A::error(te, nf, p) : A::error_inside(nf, p);
                        if (!(E <= T(1))) return;
                        const int x = ax ? s : c, y = ax ? c : s;
                        table.add((unsigned)y * (unsigned)W + (unsigned)x,
                                  A::mul(a.max_val, A::template profile_tab<K>(A::sqrt(E), gtab)));
                    };
                    if (sc >= 0 && sc <= s_hi) pixel(te_c, ne_c, sc);
                    /* the upward and downward span walks, one step of each per level */
                    T tu = te_c, nu = ne_c, td = te_c, nd = ne_c;
                    bool up = true, dn = true;
                    for (int k = 1;; k++) {
                        tu = A::add(tu, ts);
                        nu = A::add(nu, ns);
                        td = A::sub(td, ts);
                        nd = A::sub(nd, ns);
                        const int su = sc + k, sd = sc - k;
                        up = up && fabs(nu) < thr && su <= s_hi;
                        dn = dn && fabs(nd) < thr && sd >= 0;
                        if (!(up || dn)) break;
                        if (up && su >= 0) pixel(tu, nu, su);
                        if (dn && sd <= s_hi) pixel(td, nd, sd);
                    }
                }
                __syncthreads();
            }
            /* merge the claimed slots (or, for a full pass, only reset them) */
            const bool full = s_full != 0;
            const int n = min(s_count, kSize);
            T *dst = a.out + (long long)a.frame_of_term[t] * frame_px;
            for (int i = tid; i < n; i += kTerm2Threads) {
                const int h = s_claimed[i];
                if (!full) {
                    if (OUT_MAX) global_combine_max(dst + s_key[h], s_val[h]);
                    else atomicAdd(dst + s_key[h], s_val[h]);
                }
                s_key[h] = kNoPixel;
                s_val[h] = T(0);
            }
            __syncthreads();
            if (tid == 0) {
                s_depth--;
                if (full) {
                    /* too many pixels in this partition: redo it in two halves */
                    if (lg < 24 && s_depth + 2 <= kTerm2Stack) {
                        s_stack[s_depth++] = ((part + (1u << lg)) << 5) | (lg + 1);
                        s_stack[s_depth++] = (part << 5) | (lg + 1);
                    } else {
                        atomicOr(&a.st->flags, 1 << CBC_ERR_CAPACITY);
                    }
                }
                s_count = 0;
                s_full = 0;
            }
            __syncthreads();
        }
    }
}

template <typename T, int K, int IN_MAX, int OUT_MAX>
cudaError_t launch_terms2(const Term2Args<T> &ta, cudaStream_t s)
{
    auto fn = term_render2_kernel<T, K, IN_MAX, OUT_MAX>;
    constexpr size_t smem = term2_smem<T>();
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
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kTerm2Threads, smem);
        g = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
        grid_cache[dev & 63].store(g, std::memory_order_relaxed);
    }
    const long long grid = ta.n_terms < g ? ta.n_terms : g;
    if (grid < 1) return cudaSuccess;
    fn<<<(unsigned)grid, kTerm2Threads, smem, s>>>(ta);
    note_launches(1);
    return cudaGetLastError();
}

template <typename T, int K>
cudaError_t launch_terms2_k(const Term2Args<T> &ta, int mode, cudaStream_t s)
{
    return mode == kAccMaxSum ? launch_terms2<T, K, 1, 0>(ta, s) : launch_terms2<T, K, 0, 1>(ta, s);
}

template <typename T>
int accumulate_impl(T *out, long long n_frames, long long H, long long W, const T *lines,
                    long long n_lines, const void *terms, int term_bytes, const void *frames,
                    int frame_bytes, long long n_terms, T max_val, int kernel, int in_overlap,
                    int out_overlap, void *workspace, size_t ws_bytes, long long ck_capacity,
                    long long table_capacity, void *stream)
{
    clear_error();
    if (n_frames < 0 || H < 0 || W < 0 || n_lines < 0 || n_terms < 0)
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
    if (H * W > (long long)UINT_MAX) return fail(CBC_ERR_INVALID, "frames larger than 2^32 pixels");
    if (ck_capacity < 0 || ck_capacity > INT_MAX)
        return fail(CBC_ERR_INVALID, "checkpoint_capacity out of range");
    const int mode = (in_overlap == CBC_MAX ? 1 : 0) | (out_overlap == CBC_MAX ? 2 : 0);
    const bool table = mode == kAccMaxSum || mode == kAccSumMax;
    if (table && (table_capacity < 0 || (table_capacity & (table_capacity - 1))))
        return fail(CBC_ERR_INVALID, "table_capacity must be 0 or a power of two");
    if (!table) table_capacity = 0;
    const long long pixels = n_frames * H * W;
    if (n_lines > 0 && pixels > 0 && !out) return fail(CBC_ERR_INVALID, "null pointer");
    AccLayout L = acc_layout(n_lines, n_terms, ck_capacity, table_capacity, sizeof(LineRec<T>),
                             sizeof(Checkpoint<T>), sizeof(T));
    if (!workspace || ws_bytes < L.total)
        return fail(CBC_ERR_INVALID, "workspace too small (" + std::to_string(ws_bytes) + " < " +
                                         std::to_string(L.total) + ")");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    DevStatus *st = reinterpret_cast<DevStatus *>(ws + L.status);
    int *frame_of_line = reinterpret_cast<int *>(ws + L.frame_of_line);
    int *term_of_line = reinterpret_cast<int *>(ws + L.term_of_line);
    int *frame_of_term = reinterpret_cast<int *>(ws + L.frame_of_term);
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(ws + L.keys);
    T *vals = reinterpret_cast<T *>(ws + L.vals);

    init_status_kernel<<<1, 1, 0, s>>>(st, CBC_STRATEGY_LINES);
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = launch_frames_check(frames, frame_bytes, n_terms, n_frames, frame_of_term, st, s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (n_lines == 0 || pixels == 0) return CBC_OK;
    const unsigned nb = (unsigned)((n_lines + kThreads - 1) / kThreads);
    e = launch_term_frames(terms, term_bytes, frame_of_term, n_lines, n_terms, term_of_line,
                           frame_of_line, st, s);
    if (e == cudaSuccess && table && table_capacity > 0)
        e = clear_table(keys, vals, table_capacity, s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    Geometry g;
    g.H = (int)H;
    g.W = (int)W;
    g.tile_w = g.tile_h = kDefaultTileW;
    g.tiles_x = g.tiles_y = 1;
    LineRec<T> *recs = reinterpret_cast<LineRec<T> *>(ws + L.recs);
    Checkpoint<T> *cks = reinterpret_cast<Checkpoint<T> *>(ws + L.cks);
    prep_kernel<T, int32_t, false, true><<<nb, kThreads, 0, s>>>(
        lines, frame_of_line, n_lines, n_frames, g, recs, nullptr, cks, ck_capacity, st, nullptr);
    note_launches(1);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    int *tcount = reinterpret_cast<int *>(ws + L.tcount);
    int *toff = reinterpret_cast<int *>(ws + L.toff);
    int *tfill = reinterpret_cast<int *>(ws + L.tfill);
    float *test = reinterpret_cast<float *>(ws + L.test);
    int *tlines = reinterpret_cast<int *>(ws + L.tlines);
    int *tbig = reinterpret_cast<int *>(ws + L.tbig);
    unsigned long long *cursor = reinterpret_cast<unsigned long long *>(ws + L.counters);
    int *nbig = reinterpret_cast<int *>(ws + L.counters + 8);
    float *big_est = reinterpret_cast<float *>(ws + L.counters + 12);
    if (table) {
        /* per term: its drawable lines, a pixel estimate, and the table / shared split */
        e = cudaMemsetAsync(tcount, 0, sizeof(int) * (size_t)n_terms, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(test, 0, sizeof(float) * (size_t)n_terms, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(ws + L.counters, 0, 16, s);
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
        const unsigned nbt = (unsigned)((n_terms + kThreads - 1) / kThreads);
        term_count2_kernel<T><<<nb, kThreads, 0, s>>>(recs, term_of_line, n_lines, tcount, test);
        term_offsets_kernel<<<nbt, kThreads, 0, s>>>(tcount, toff, tfill, n_terms, cursor);
        term_fill2_kernel<T><<<nb, kThreads, 0, s>>>(recs, term_of_line, n_lines, tfill, tlines);
        term_class_kernel<<<nbt, kThreads, 0, s>>>(
            tcount, test, n_terms,
            (float)kTerm2MaxParts * kTerm2Fill * (float)(1 << Term2Table<T>::kBits), tbig, nbig,
            big_est);
        note_launches(4);
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    }
    AccArgs<T> a;
    a.d.recs = recs;
    a.d.cks = cks;
    a.d.H = (int)H;
    a.d.W = (int)W;
    a.d.st = st;
    a.d.work = &st->work;
    a.out = out;
    a.max_val = max_val;
    a.term_of_line = term_of_line;
    a.keys = keys;
    a.vals = vals;
    a.mask = table_capacity > 0 ? (unsigned long long)table_capacity - 1ull : 0ull;
    a.tbig = tbig;
    a.nbig = nbig;
    a.big_est = big_est;
    a.table_capacity = table_capacity;
    switch (kernel) {
    case CBC_BIWEIGHT:    e = launch_accumulate<T, CBC_BIWEIGHT>(a, mode, s); break;
    case CBC_GAUSSIAN:    e = launch_accumulate<T, CBC_GAUSSIAN>(a, mode, s); break;
    case CBC_PARABOLIC:   e = launch_accumulate<T, CBC_PARABOLIC>(a, mode, s); break;
    case CBC_RECTANGULAR: e = launch_accumulate<T, CBC_RECTANGULAR>(a, mode, s); break;
    default:              e = launch_accumulate<T, CBC_TRIANGULAR>(a, mode, s); break;
    }
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (table) {
        /* the other terms in shared memory, then the table's terms merged */
        Term2Args<T> ta{recs, cks, st, out, max_val, (int)H, (int)W, tcount, toff, tlines, tbig,
                        frame_of_term, test, n_terms};
        switch (kernel) {
        case CBC_BIWEIGHT:    e = launch_terms2_k<T, CBC_BIWEIGHT>(ta, mode, s); break;
        case CBC_GAUSSIAN:    e = launch_terms2_k<T, CBC_GAUSSIAN>(ta, mode, s); break;
        case CBC_PARABOLIC:   e = launch_terms2_k<T, CBC_PARABOLIC>(ta, mode, s); break;
        case CBC_RECTANGULAR: e = launch_terms2_k<T, CBC_RECTANGULAR>(ta, mode, s); break;
        default:              e = launch_terms2_k<T, CBC_TRIANGULAR>(ta, mode, s); break;
        }
        if (e == cudaSuccess && table_capacity > 0)
            e = launch_merge(out, keys, vals, table_capacity, frame_of_term, H * W,
                             mode == kAccSumMax, st, s);
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    }
    return CBC_OK;
}

}  // namespace cbc

extern "C" {

size_t cbc_accumulate_lines_workspace_size(int64_t n_lines, int64_t n_terms,
                                           int64_t checkpoint_capacity, int64_t table_capacity,
                                           int32_t elem_bytes)
{
    if (n_lines < 0 || n_terms < 0 || checkpoint_capacity < 0 || table_capacity < 0 ||
        (elem_bytes != 4 && elem_bytes != 8))
        return 0;
    const size_t rec = elem_bytes == 4 ? sizeof(cbc::LineRec<float>) : sizeof(cbc::LineRec<double>);
    const size_t ck = elem_bytes == 4 ? sizeof(cbc::Checkpoint<float>) : sizeof(cbc::Checkpoint<double>);
    return cbc::acc_layout(n_lines, n_terms, checkpoint_capacity, table_capacity, rec, ck,
                           (size_t)elem_bytes).total;
}

int cbc_accumulate_lines_f32(float *out, int64_t n_frames, int64_t height, int64_t width,
                             const float *lines, int64_t n_lines, const void *terms,
                             int32_t term_bytes, const void *frames, int32_t frame_bytes,
                             int64_t n_terms, float max_val, int32_t kernel, int32_t in_overlap,
                             int32_t out_overlap, void *workspace, size_t workspace_bytes,
                             int64_t checkpoint_capacity, int64_t table_capacity, void *stream)
{
    return cbc::accumulate_impl<float>(out, n_frames, height, width, lines, n_lines, terms,
                                       term_bytes, frames, frame_bytes, n_terms, max_val, kernel,
                                       in_overlap, out_overlap, workspace, workspace_bytes,
                                       checkpoint_capacity, table_capacity, stream);
}

int cbc_accumulate_lines_f64(double *out, int64_t n_frames, int64_t height, int64_t width,
                             const double *lines, int64_t n_lines, const void *terms,
                             int32_t term_bytes, const void *frames, int32_t frame_bytes,
                             int64_t n_terms, double max_val, int32_t kernel, int32_t in_overlap,
                             int32_t out_overlap, void *workspace, size_t workspace_bytes,
                             int64_t checkpoint_capacity, int64_t table_capacity, void *stream)
{
    return cbc::accumulate_impl<double>(out, n_frames, height, width, lines, n_lines, terms,
                                        term_bytes, frames, frame_bytes, n_terms, max_val, kernel,
                                        in_overlap, out_overlap, workspace, workspace_bytes,
                                        checkpoint_capacity, table_capacity, stream);
}

}  // extern "C"
