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
 * Lines strategy (the default; one stream, no host synchronisation):
 *   1. prep_kernel   one thread per line: frame index check, walk parameters
 *                    (LineRec), checkpoint block, the list of long walks.
 *   2. walk_ordered_kernel  one thread per line, long walks first: the exact walk
 *                    state every 16 in-frame columns (walk checkpoints).
 *   3. segments_kernel  persistent: warps take 32 (line, 8-column segment) items,
 *                    replay the walks from their checkpoints, queue the visited
 *                    pixels in per-warp rings and evaluate them on full warps, one
 *                    L2 reduction per drawn pixel (drive_segments, cbc_common.cuh).
 * Tiles strategy (on request):
 *   1. prep_kernel   as above, plus conservative tile coverage -> per-bin counts.
 *   2. offsets_kernel  block scan of the per-bin counts, one atomic per block ->
 *                    bin offsets into the pair buffer (a counting sort on the
 *                    (frame, tile) key), capacity check.
 *   3. fill_kernel   one thread per line: line id into each of its bins.
 *   4. render_kernel one CTA per (frame, tile) bin with lines: stage the output tile
 *                    in shared memory, replay each line's walk to the tile's columns
 *                    (one thread per line), then evaluate the spans of all
 *                    (line, column) entries in parallel with shared-memory atomics,
 *                    write the tile back once.  Empty bins are never touched.
 * Host frames (cbc_draw_lines_host_*): the lines strategy into a device scratch at
 * the overlap's identity, then combine_host_kernel merges the drawn pixels into the
 * host frames over NVLink-C2C.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <limits.h>
#include <stdio.h>
#include <string.h>
#include <cstring>
#include <string>
#include <atomic>
#include <mutex>
#include <vector>

#include "cbc_common.cuh"

#define CBC_VERSION "cbclib_v2_gb300 0.1.0 (sm_103a)"

namespace cbc {

template <typename T>
struct RenderArgs {
    T *out;
    const LineRec<T> *recs;
    const int *counts;
    const int *offsets;
    const int *pairs;
    const Checkpoint<T> *cks;
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
           (size_t)ent_cap + kMaxChunk * sizeof(SlotParams<T>) +
           kMaxChunk * sizeof(WalkSlot<T>) + 4 * sizeof(int) + 64;
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
    const int npix = tw * th;

    T *acc = reinterpret_cast<T *>(smem);
    Entry<T> *ent = reinterpret_cast<Entry<T> *>(acc + (size_t)g.tile_w * g.tile_h);
    SlotParams<T> *prm = reinterpret_cast<SlotParams<T> *>(ent + a.ent_cap);
    WalkSlot<T> *wsl = reinterpret_cast<WalkSlot<T> *>(prm + kMaxChunk);
    int *totals = reinterpret_cast<int *>(wsl + kMaxChunk);          /* entries, segments */
    unsigned char *eslot = reinterpret_cast<unsigned char *>(totals + 4);

    const T init = OV == CBC_SUM ? Sentinel<T>::sum() : T(-INFINITY);
    for (int e = threadIdx.x; e < npix; e += blockDim.x) acc[e] = init;

    const int *seg = a.pairs + a.offsets[bin];
    for (int cb = 0; cb < cnt; cb += a.chunk) {
        const int n = min(a.chunk, cnt - cb);
        /* phase A: per-line parameters, in-tile walk-index range, segment count */
        if (threadIdx.x < 32) {
            int my_count = 0, my_nseg = 0;
            if ((int)threadIdx.x < n) {
                const LineRec<T> r = a.recs[seg[cb + threadIdx.x]];
                const int ax = r.flags & kAxisY;
                const int sx = (r.flags & kStepXNeg) ? -1 : 1, sy = (r.flags & kStepYNeg) ? -1 : 1;
                const int sa = ax ? sy : sx;
                const int la0 = ax ? y0 : x0, la1 = ax ? y0 + th - 1 : x0 + tw - 1;
                int k_lo = sa > 0 ? la0 - r.c0 : r.c0 - la1;
                int k_hi = sa > 0 ? la1 - r.c0 : r.c0 - la0;
                k_lo = max(k_lo, 0);
                k_hi = min(k_hi, r.ncols - 1);
                my_count = max(0, k_hi - k_lo + 1);
                my_nseg = my_count > 0 ? k_hi / kCkCols - k_lo / kCkCols + 1 : 0;
                SlotParams<T> p;
                p.ts = ax ? r.t0 : r.t1;              /* d te / d short */
                p.ns = ax ? r.t1 : -r.t0;             /* d ne / d short: normal = (t1, -t0) */
                p.len = r.len;
                p.len2 = r.len2;
                p.ww = r.ww;
                p.rlen = r.rlen;
                p.rww = r.rww;
                p.ne_thr = r.ne_thr;
                p.rns = 1.0f / (float)p.ns;
                p.ss = ax ? sx : sy;
                p.axis = ax;
                p.fast = (r.flags & kFastDiv) ? 1 : 0;
                prm[threadIdx.x] = p;
                WalkSlot<T> w;
                w.sx = sx;
                w.sy = sy;
                w.d0t = sx > 0 ? r.t0 : -r.t0;
                w.d1t = sy > 0 ? r.t1 : -r.t1;
                w.d0n = sx > 0 ? r.t1 : -r.t1;
                w.d1n = sy > 0 ? -r.t0 : r.t0;
                w.x1 = r.x1;
                w.y1 = r.y1;
                w.c0 = r.c0;
                w.sa = sa;
                w.k_lo = k_lo;
                w.k_hi = k_hi;
                w.ck_base = r.ck_base;
                w.axis = ax;
                wsl[threadIdx.x] = w;
            }
            int ic = my_count, is = my_nseg;
            for (int o = 1; o < 32; o <<= 1) {
                int u = __shfl_up_sync(0xffffffffu, ic, o);
                int v = __shfl_up_sync(0xffffffffu, is, o);
                if ((int)threadIdx.x >= o) { ic += u; is += v; }
            }
            if ((int)threadIdx.x < n) {
                wsl[threadIdx.x].ent_base = ic - my_count;
                wsl[threadIdx.x].seg_base = is - my_nseg;
            }
            if (threadIdx.x == 31) { totals[0] = ic; totals[1] = is; }
        }
        __syncthreads();
        const int total = totals[0], nsegs = totals[1];
        for (int e = threadIdx.x; e < total; e += blockDim.x) ent[e].c = kInvalidEntry;
        __syncthreads();

        /* phase B: every (line, kCkCols-column segment) resumes the walk (bresenham.hpp:
         * 352-383 outer loop) from its checkpoint, one thread each, and records the
         * filled columns inside the tile */
        for (int it = threadIdx.x; it < nsegs; it += blockDim.x) {
            int sl = 0;
            #pragma unroll
            for (int bit = 16; bit > 0; bit >>= 1)
                if (sl + bit < n && wsl[sl + bit].seg_base <= it) sl += bit;
            const WalkSlot<T> &w = wsl[sl];
            const int sg = w.k_lo / kCkCols + (it - w.seg_base);
            const Checkpoint<T> ck = a.cks[w.ck_base + sg];
            if (ck.cx == INT_MIN) continue;
            const int lo = max(sg * kCkCols, w.k_lo), hi = min(sg * kCkCols + kCkCols - 1, w.k_hi);
            Walker<T> wk;
            wk.sx = w.sx;
            wk.sy = w.sy;
            wk.d0t = w.d0t;
            wk.d1t = w.d1t;
            wk.d0n = w.d0n;
            wk.d1n = w.d1n;
            wk.cx = ck.cx;
            wk.cy = ck.cy;
            wk.te = ck.te;
            wk.ne = ck.ne;
            int guard = 0;
            while (wk.cx != w.x1 && wk.cy != w.y1) {
                const typename Walker<T>::Next mv = wk.decide();
                const int c = w.axis ? wk.cy : wk.cx;
                const int idx = (c - w.c0) * w.sa;
                if (w.axis ? mv.ny : mv.nx) {
                    if (idx >= lo && idx <= hi) {
                        const int k = w.ent_base + (idx - w.k_lo);
                        Entry<T> en;
                        en.c = c;
                        en.sc = w.axis ? wk.cx : wk.cy;
                        en.te = wk.te;
                        en.ne = wk.ne;
                        ent[k] = en;
                        eslot[k] = (unsigned char)sl;
                        if (idx == hi) break;
                    }
                }
                if (idx > hi) break;
                wk.step(mv);
                if (++guard > 4 * CBC_MAX_WALK + 64) {
                    atomicOr(&a.st->flags, 1 << CBC_ERR_RANGE);
                    break;
                }
            }
        }
        __syncthreads();

        /* phase C: the centre and both span halves of every entry (bresenham.hpp:364-381).
         * Each warp flattens 32 entries into (entry, short offset j) items, one pixel
         * per lane.  Pixel j != 0 lies |j| span steps from the centre: its errors are
         * |j| sequential additions, and it is visited iff the first and the |j|-th
         * step both pass the span test (the passing steps form an interval, because
         * ne is monotone along a span and the test is a threshold on |ne|). */
        {
            const int lane = threadIdx.x & 31;
            const int nwarps = blockDim.x >> 5;
            for (int e0 = (threadIdx.x >> 5) * 32; e0 < total; e0 += nwarps * 32) {
                const int e = e0 + lane;
                int cnt = 0, jlo = 0;
                if (e < total) {
                    const Entry<T> en = ent[e];
                    if (en.c != kInvalidEntry) {
                        const SlotParams<T> &p = prm[eslot[e]];
                        const int s_lo = p.axis ? x0 : y0, s_hi = p.axis ? x0 + tw - 1 : y0 + th - 1;
                        cnt = span_window(p, en.sc, en.ne, s_lo, s_hi, jlo);
                    }
                }
                int incl = cnt;
                for (int o = 1; o < 32; o <<= 1) {
                    int u = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += u;
                }
                const int excl = incl - cnt;
                const int items = __shfl_sync(0xffffffffu, incl, 31);
                for (int t0 = 0; t0 < items; t0 += 32) {
                    const int t = t0 + lane;
                    int o = 0;
                    #pragma unroll
                    for (int bit = 16; bit > 0; bit >>= 1) {
                        const int v = __shfl_sync(0xffffffffu, excl, o + bit);
                        if (v <= t) o += bit;
                    }
                    const int off_o = __shfl_sync(0xffffffffu, excl, o);
                    const int jlo_o = __shfl_sync(0xffffffffu, jlo, o);
                    if (t >= items) continue;
                    const Entry<T> en = ent[e0 + o];
                    const SlotParams<T> &p = prm[eslot[e0 + o]];
                    const int j = jlo_o + (t - off_o);
                    T te = en.te, ne = en.ne;
                    bool visited = true;
                    if (j != 0) {
                        const T dt = j > 0 ? p.ts : -p.ts, dn = j > 0 ? p.ns : -p.ns;
                        te = A::add(te, dt);
                        ne = A::add(ne, dn);
                        visited = fabs(ne) < p.ne_thr;
                        const int k = j > 0 ? j : -j;
                        for (int i = 1; i < k; i++) {
                            te = A::add(te, dt);
                            ne = A::add(ne, dn);
                        }
                        visited = visited && fabs(ne) < p.ne_thr;
                    }
                    if (!visited) continue;
                    const T nf = A::nterm(ne, p);
                    const T E = A::error(te, nf, p);
                    if (!(E <= T(1))) continue;
                    const T v = A::mul(a.max_val, A::template profile<K>(A::sqrt(E)));
                    const int y = en.sc + j;
                    T *dst = p.axis ? acc + ((ptrdiff_t)(en.c - y0) * tw + (y - x0))
                                    : acc + ((ptrdiff_t)(y - y0) * tw + (en.c - x0));
                    if (OV == CBC_SUM) atomicAdd(dst, v); else combine_max(dst, v);
                }
            }
        }
        __syncthreads();
    }

    /* sparse read-modify-write: only pixels that some line drew are read and written;
     * each thread scans a group of 4 pixels of one tile row per step */
    T *gout = a.out + ((size_t)frame * g.H + y0) * g.W + x0;
    const int gpr = (tw + 3) >> 2;                       /* 4-pixel groups per row */
    for (int q = threadIdx.x; q < gpr * th; q += blockDim.x) {
        const int r = q / gpr, c = (q - r * gpr) * 4;
        const T *src = acc + (size_t)r * tw + c;
        T *dst = gout + (size_t)r * g.W + c;
        const int m = min(4, tw - c);
        #pragma unroll
        for (int k = 0; k < 4; k++) {
            if (k >= m) break;
            const T v = src[k];
            if (OV == CBC_SUM) {
                if (Sentinel<T>::sum_touched(v)) dst[k] = A::add(dst[k], v);
            } else if (v != T(-INFINITY)) {
                const T o = dst[k];
                if (o < v) dst[k] = v;
            }
        }
    }
}

/* ---- lines strategy ----------------------------------------------------------------
 * drive_segments (cbc_common.cuh) enumerates the drawn pixels; the forward action
 * evaluates the profile and combines each value into `out` with an L2 reduction. */

template <typename T, int K, int OV>
struct ForwardAct {
    static constexpr bool kNeedsError = true;
    T *out;
    T max_val;
    int W;
    const float *gtab;   /* gaussian table (shared-memory copy) */
    struct Pre {};
    template <class ST>
    __device__ __forceinline__ void item_begin(int, const ST &) {}
    __device__ __forceinline__ void item_end(int, const SlotTable<T> &) {}
    __device__ __forceinline__ Pre prefetch(const SlotTable<T> &, int, int, int) const { return {}; }
    __device__ __forceinline__ void pixel(const SlotTable<T> &S, int slot, int px, int py, T E,
                                          T, T, Pre) {
        using A = Ar<T>;
        const T v = A::mul(max_val, A::template profile_tab<K>(A::sqrt(E), gtab));
        T *dst = out + S.fbase[slot] + (long long)py * W + px;
        if (OV == CBC_SUM) atomicAdd(dst, v); else global_combine_max(dst, v);
    }
};

/* max overlap into frames that start at zero, keeping each pixel's winner: the value's
 * bits (positive floats order as integers) over the complement of the line index, so
 * one 64-bit atomicMax keeps the largest value and, among equal values, the smallest
 * line, which is the line sequential std::max keeps (bresenham.cpp:71) */
template <int K>
struct PackedMaxAct {
    static constexpr bool kNeedsError = true;
    unsigned long long *packed;
    float max_val;
    int W;
    const float *gtab;
    struct Pre {};
    template <class ST>
    __device__ __forceinline__ void item_begin(int, const ST &) {}
    __device__ __forceinline__ void item_end(int, const SlotTable<float> &) {}
    __device__ __forceinline__ Pre prefetch(const SlotTable<float> &, int, int, int) const {
        return {};
    }
    __device__ __forceinline__ void pixel(const SlotTable<float> &S, int slot, int px, int py,
                                          float E, float, float, Pre) {
        using A = Ar<float>;
        const float v = A::mul(max_val, A::template profile_tab<K>(A::sqrt(E), gtab));
        if (!(v > 0.0f)) return;      /* std::max(0, v) keeps the zero */
        const unsigned long long key =
            ((unsigned long long)__float_as_uint(v) << 32) |
            (unsigned long long)(0xffffffffu - (unsigned)S.line[slot]);
        atomicMax(packed + S.fbase[slot] + (long long)py * W + px, key);
    }
};

struct PackedArgs {
    DriveArgs<float> d;
    unsigned long long *packed;
    float max_val;
};

template <int K>
__global__ void __launch_bounds__(kSegWarps * 32, kSegMinBlocks)
packed_max_kernel(PackedArgs a)
{
    PackedMaxAct<K> act;
    act.packed = a.packed;
    act.max_val = a.max_val;
    act.W = a.d.W;
    act.gtab = stage_gauss_table<float, K>();
    drive_segments(a.d, act);
}

/* packed -> frames and winners; packed is left zero for the next call */
static __global__ void __launch_bounds__(kThreads)
unpack_max_kernel(unsigned long long *__restrict__ packed, float *__restrict__ out,
                  int *__restrict__ winner, long long n, const DevStatus *st)
{
    if (st->flags & kFatal) return;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long k = packed[i];
        const unsigned hi = (unsigned)(k >> 32);
        out[i] = __uint_as_float(hi);
        winner[i] = hi ? (int)(0xffffffffu - (unsigned)k) : 0x7f7f7f7f;
        if (k) packed[i] = 0ull;
    }
}

template <typename T>
struct SegArgs {
    DriveArgs<T> d;
    T *out;
    T max_val;
};

template <typename T, int K, int OV>
__global__ void __launch_bounds__(kSegWarps * 32, kSegMinBlocks)
segments_kernel(SegArgs<T> a)
{
    ForwardAct<T, K, OV> act;
    act.out = a.out;
    act.max_val = a.max_val;
    act.W = a.d.W;
    act.gtab = stage_gauss_table<T, K>();
    drive_segments(a.d, act);
}

/* ---- host side ----------------------------------------------------------------- */

thread_local std::string g_error;

int fail(int code, const std::string &msg)
{
    g_error = msg;
    return code;
}

void clear_error() { g_error.clear(); }

std::atomic<int> g_launches{0};

void note_launches(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

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

struct Layout {
    size_t status, recs, counts, offsets, fillpos, pairs, cks, frames, longs, total;
};

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct Resolved {
    int tile_w, tile_h, chunk, ent_cap, threads, strategy;
};

bool resolve_tuning(const cbc_tuning *t, Resolved &r, std::string &why)
{
    r.tile_w = (t && t->tile_w) ? t->tile_w : kDefaultTileW;
    r.tile_h = (t && t->tile_h) ? t->tile_h : kDefaultTileH;
    r.chunk = (t && t->chunk_lines) ? t->chunk_lines : kDefaultChunk;
    r.threads = (t && t->threads) ? t->threads : kThreads;
    r.strategy = t ? t->strategy : CBC_STRATEGY_AUTO;
    if (r.strategy < CBC_STRATEGY_AUTO || r.strategy > CBC_STRATEGY_LINES) {
        why = "strategy must be CBC_STRATEGY_AUTO, _TILES or _LINES";
        return false;
    }
    if (r.threads != 128 && r.threads != 256) { why = "threads must be 128 or 256"; return false; }
    if (r.tile_w < 16 || r.tile_w > 256 || (r.tile_w & 3)) { why = "tile_w must be a multiple of 4 in [16, 256]"; return false; }
    if (r.tile_h < 4 || r.tile_h > 256) { why = "tile_h must be in [4, 256]"; return false; }
    if (r.chunk < 1 || r.chunk > kMaxChunk) { why = "chunk_lines must be in [1, 32]"; return false; }
    r.ent_cap = r.chunk * (r.tile_w > r.tile_h ? r.tile_w : r.tile_h);
    return true;
}

Layout make_layout(long long n_frames, long long H, long long W, long long n_lines,
                   long long capacity, long long ck_capacity, size_t rec_bytes,
                   size_t ck_bytes, const Resolved &t)
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
    L.cks = off;     off = align_up(off + ck_bytes * (size_t)ck_capacity, 256);
    L.frames = off;  off = align_up(off + sizeof(int) * (size_t)n_lines, 256);
    L.longs = off;   off = align_up(off + sizeof(int) * (size_t)n_lines, 256);
    L.total = off;
    return L;
}

template <typename T, int K, int OV>
cudaError_t launch_render(const RenderArgs<T> &ra, long long n_bins, size_t smem, cudaStream_t s,
                          int threads)
{
    auto fn = render_kernel<T, K, OV>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    fn<<<(unsigned)n_bins, threads, smem, s>>>(ra);
    note_launches(1);
    return cudaGetLastError();
}

template <typename T, int K>
cudaError_t launch_render_ov(const RenderArgs<T> &ra, int overlap, long long n_bins, size_t smem,
                             cudaStream_t s, int threads)
{
    return overlap == CBC_MAX ? launch_render<T, K, CBC_MAX>(ra, n_bins, smem, s, threads)
                              : launch_render<T, K, CBC_SUM>(ra, n_bins, smem, s, threads);
}

template <typename T>
cudaError_t launch_render_k(const RenderArgs<T> &ra, int kernel, int overlap, long long n_bins,
                            size_t smem, cudaStream_t s, int threads)
{
    switch (kernel) {
    case CBC_BIWEIGHT:    return launch_render_ov<T, CBC_BIWEIGHT>(ra, overlap, n_bins, smem, s, threads);
    case CBC_GAUSSIAN:    return launch_render_ov<T, CBC_GAUSSIAN>(ra, overlap, n_bins, smem, s, threads);
    case CBC_PARABOLIC:   return launch_render_ov<T, CBC_PARABOLIC>(ra, overlap, n_bins, smem, s, threads);
    case CBC_RECTANGULAR: return launch_render_ov<T, CBC_RECTANGULAR>(ra, overlap, n_bins, smem, s, threads);
    default:              return launch_render_ov<T, CBC_TRIANGULAR>(ra, overlap, n_bins, smem, s, threads);
    }
}

template <typename T, int K, int OV>
cudaError_t launch_segments(const SegArgs<T> &sa, cudaStream_t s)
{
    /* persistent grid: every CTA that fits at once, no more */
    const unsigned grid = resident_grid(segments_kernel<T, K, OV>, kSegWarps * 32);
    segments_kernel<T, K, OV><<<grid, kSegWarps * 32, 0, s>>>(sa);
    note_launches(1);
    return cudaGetLastError();
}

template <typename T, int K>
cudaError_t launch_segments_ov(const SegArgs<T> &sa, int overlap, cudaStream_t s)
{
    return overlap == CBC_MAX ? launch_segments<T, K, CBC_MAX>(sa, s)
                              : launch_segments<T, K, CBC_SUM>(sa, s);
}

template <typename T>
cudaError_t launch_segments_k(const SegArgs<T> &sa, int kernel, int overlap, cudaStream_t s)
{
    switch (kernel) {
    case CBC_BIWEIGHT:    return launch_segments_ov<T, CBC_BIWEIGHT>(sa, overlap, s);
    case CBC_GAUSSIAN:    return launch_segments_ov<T, CBC_GAUSSIAN>(sa, overlap, s);
    case CBC_PARABOLIC:   return launch_segments_ov<T, CBC_PARABOLIC>(sa, overlap, s);
    case CBC_RECTANGULAR: return launch_segments_ov<T, CBC_RECTANGULAR>(sa, overlap, s);
    default:              return launch_segments_ov<T, CBC_TRIANGULAR>(sa, overlap, s);
    }
}

/* CSR frame offsets -> one int32 frame index per line (binary search), with the
 * offsets' rules checked on the device */
__global__ void __launch_bounds__(kThreads)
csr_frames_kernel(const int64_t *__restrict__ offs, long long n_frames, long long n_lines,
                  int *__restrict__ frames, DevStatus *st)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= n_frames) {
        const long long o = offs[i];
        bool bad = (i == 0 && o != 0) || (i == n_frames && o != n_lines) ||
                   (i < n_frames && offs[i + 1] < o);
        if (bad) {
            atomicOr(&st->flags, 1 << CBC_ERR_INDEX);
            atomicMin(&st->bad_line, (unsigned long long)i);
        }
    }
    if (i >= n_lines) return;
    long long lo = 0, hi = n_frames;          /* last f with offs[f] <= i */
    while (hi - lo > 1) {
        const long long mid = (lo + hi) >> 1;
        if (offs[mid] <= i) lo = mid; else hi = mid;
    }
    frames[i] = (int)lo;
}


template <typename T>
int draw_lines_impl(T *out, long long n_frames, long long H, long long W, const T *lines,
                    long long n_lines, const void *idxs, int idx_bytes, T max_val, int kernel,
                    int overlap, void *workspace, size_t ws_bytes, long long capacity,
                    long long ck_capacity, const cbc_tuning *tuning, void *stream,
                    const int64_t *csr = nullptr, unsigned long long *packed = nullptr,
                    int *winner = nullptr)
{
    g_error.clear();
    if (n_frames < 0 || H < 0 || W < 0 || n_lines < 0)
        return fail(CBC_ERR_INVALID, "negative size");
    if (H > INT_MAX / 2 || W > INT_MAX / 2)
        return fail(CBC_ERR_INVALID, "frame dimensions must be below 2^30");
    if (n_frames > INT_MAX)     /* line records hold the frame as a 32-bit index */
        return fail(CBC_ERR_INVALID, "n_frames must not exceed 2^31 - 1");
    if (kernel < 0 || kernel > 4) return fail(CBC_ERR_INVALID, "Invalid kernel type");
    if (overlap != CBC_SUM && overlap != CBC_MAX)
        return fail(CBC_ERR_INVALID, "Invalid overlap keyword");
    if (idxs && idx_bytes != 4 && idx_bytes != 8)
        return fail(CBC_ERR_INVALID, "idx_bytes must be 4 or 8");
    if (!idxs && !csr && n_lines > 0 && n_frames != 1 && n_frames != n_lines)
        return fail(CBC_ERR_INVALID, "idxs has an incompatible size (" + std::to_string(n_lines) +
                                         " != " + std::to_string(n_frames) + ")");
    if (n_lines > 0 && ((!out && !packed) || !lines) && n_frames * H * W > 0)
        return fail(CBC_ERR_INVALID, "null pointer");
    if (capacity < 0 || capacity > INT_MAX) return fail(CBC_ERR_INVALID, "pair_capacity out of range");
    if (ck_capacity < 0 || ck_capacity > INT_MAX)
        return fail(CBC_ERR_INVALID, "checkpoint_capacity out of range");
    if (n_lines > INT_MAX) return fail(CBC_ERR_INVALID, "too many lines");
    Resolved t;
    std::string why;
    if (!resolve_tuning(tuning, t, why)) return fail(CBC_ERR_INVALID, why);
    Layout L = make_layout(n_frames, H, W, n_lines, capacity, ck_capacity, sizeof(LineRec<T>),
                           sizeof(Checkpoint<T>), t);
    if (!workspace || ws_bytes < L.total)
        return fail(CBC_ERR_INVALID, "workspace too small (" + std::to_string(ws_bytes) + " < " +
                                         std::to_string(L.total) + ")");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    DevStatus *st = reinterpret_cast<DevStatus *>(ws + L.status);
    /* the lines strategy is faster at every density measured on GB300 (1k to 95k
     * lines per megapixel, 1.2x to 3.4x); the tiles strategy runs when asked for */
    const int strategy = t.strategy == CBC_STRATEGY_TILES ? CBC_STRATEGY_TILES
                                                          : CBC_STRATEGY_LINES;
    CallTimer timer(s);
    timer.mark(0);
    init_status_kernel<<<1, 1, 0, s>>>(st, strategy);
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && csr) {
        if (n_frames > INT_MAX) return fail(CBC_ERR_INVALID, "too many frames");
        int *fr = reinterpret_cast<int *>(ws + L.frames);
        const long long m = (n_lines > n_frames ? n_lines : n_frames + 1);
        csr_frames_kernel<<<(unsigned)((m + kThreads - 1) / kThreads), kThreads, 0, s>>>(
            csr, n_frames, n_lines, fr, st);
        note_launches(1);
        e = cudaGetLastError();
        idxs = fr;
        idx_bytes = 4;
    }
    Geometry g;
    g.H = (int)H;
    g.W = (int)W;
    g.tile_w = t.tile_w;
    g.tile_h = t.tile_h;
    g.tiles_x = (int)((W + t.tile_w - 1) / t.tile_w);
    g.tiles_y = (int)((H + t.tile_h - 1) / t.tile_h);
    long long n_bins = n_frames * (long long)g.tiles_x * g.tiles_y;
    if (n_bins > INT_MAX) return fail(CBC_ERR_INVALID, "too many (frame, tile) bins");
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (n_lines == 0) return CBC_OK;
    unsigned nb_lines = (unsigned)((n_lines + kThreads - 1) / kThreads);
    LineRec<T> *recs = reinterpret_cast<LineRec<T> *>(ws + L.recs);
    Checkpoint<T> *cks = reinterpret_cast<Checkpoint<T> *>(ws + L.cks);
    const bool wide = idxs && idx_bytes == 8;
    if (strategy == CBC_STRATEGY_LINES) {
        /* records and checkpoint blocks, then the walks: the long ones first */
        int *longs = reinterpret_cast<int *>(ws + L.longs);
        if (wide) prep_kernel<T, int64_t, false, false><<<nb_lines, kThreads, 0, s>>>(
                      lines, idxs, n_lines, n_frames, g, recs, nullptr, cks, ck_capacity, st,
                      longs);
        else      prep_kernel<T, int32_t, false, false><<<nb_lines, kThreads, 0, s>>>(
                      lines, idxs, n_lines, n_frames, g, recs, nullptr, cks, ck_capacity, st,
                      longs);
        walk_ordered_kernel<T><<<2 * nb_lines, kThreads, 0, s>>>(recs, n_lines, longs, g, cks, st);
        note_launches(2);
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
        timer.mark(1);
        timer.mark(2);
        timer.mark(3);
        if (n_frames * H * W > 0 && packed) {
            if constexpr (sizeof(T) == sizeof(float)) {
                PackedArgs pa;
                pa.packed = packed;
                pa.max_val = max_val;
                pa.d.recs = reinterpret_cast<const LineRec<float> *>(recs);
                pa.d.cks = reinterpret_cast<const Checkpoint<float> *>(cks);
                pa.d.H = (int)H;
                pa.d.W = (int)W;
                pa.d.st = st;
                pa.d.work = &st->work;
                const unsigned threads = kSegWarps * 32;
#define CBC_PACKED_CASE(KK)                                                                   \
                case KK:                                                                    \
                    packed_max_kernel<KK><<<resident_grid(packed_max_kernel<KK>, threads),   \
                                            threads, 0, s>>>(pa);                           \
                    break;
                switch (kernel) {
                CBC_PACKED_CASE(CBC_BIWEIGHT)
                CBC_PACKED_CASE(CBC_GAUSSIAN)
                CBC_PACKED_CASE(CBC_PARABOLIC)
                CBC_PACKED_CASE(CBC_RECTANGULAR)
                default: CBC_PACKED_CASE(CBC_TRIANGULAR)
                }
#undef CBC_PACKED_CASE
                note_launches(1);
                if (out && winner) {      /* else the caller keeps the packed pairs */
                    const long long n = n_frames * H * W;
                    int dev = 0, sms = 0;
                    cudaGetDevice(&dev);
                    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
                    const long long most = (long long)(sms > 0 ? sms : 132) * 16;
                    long long blocks = (n + kThreads - 1) / kThreads;
                    if (blocks > most) blocks = most;
                    unpack_max_kernel<<<(unsigned)blocks, kThreads, 0, s>>>(
                        packed, reinterpret_cast<float *>(out), winner, n, st);
                    note_launches(1);
                }
                e = cudaGetLastError();
                if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
            }
        } else if (n_frames * H * W > 0) {
            SegArgs<T> sg;
            sg.out = out;
            sg.max_val = max_val;
            sg.d.recs = recs;
            sg.d.cks = cks;
            sg.d.H = (int)H;
            sg.d.W = (int)W;
            sg.d.st = st;
            sg.d.work = &st->work;
            e = launch_segments_k<T>(sg, kernel, overlap, s);
            if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
        }
        timer.mark(4);
        timer.commit();
        return CBC_OK;
    }
    int *counts = reinterpret_cast<int *>(ws + L.counts);
    if (n_bins > 0) e = cudaMemsetAsync(counts, 0, sizeof(int) * n_bins, s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (!wide)
        prep_kernel<T, int32_t, true, false><<<nb_lines, kThreads, 0, s>>>(
            lines, idxs, n_lines, n_frames, g, recs, counts, cks, ck_capacity, st, nullptr);
    else
        prep_kernel<T, int64_t, true, false><<<nb_lines, kThreads, 0, s>>>(
            lines, idxs, n_lines, n_frames, g, recs, counts, cks, ck_capacity, st, nullptr);
    note_launches(1);
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
    fill_kernel<T><<<nb_lines, kThreads, 0, s>>>(recs, n_lines, g, fillpos, pairs, capacity, cks,
                                                 st);
    note_launches(2);
    timer.mark(3);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    RenderArgs<T> ra;
    ra.out = out;
    ra.recs = recs;
    ra.counts = counts;
    ra.offsets = offsets;
    ra.pairs = pairs;
    ra.cks = cks;
    ra.st = st;
    ra.g = g;
    ra.max_val = max_val;
    ra.chunk = t.chunk;
    ra.ent_cap = t.ent_cap;
    size_t smem = render_smem_bytes<T>(t.tile_w, t.tile_h, t.ent_cap);
    e = launch_render_k<T>(ra, kernel, overlap, n_bins, smem, s, t.threads);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    timer.mark(4);
    timer.commit();
    return CBC_OK;
}

/* ---- frames in page-locked host memory ------------------------------------------
 * The lines are drawn into a device scratch that holds the overlap's identity (max:
 * -inf, which every contribution exceeds; sum: -0, which no contribution leaves
 * behind), so afterwards a scratch pixel differs from the identity exactly where
 * some line drew.  One pass then combines those pixels into the host frames through
 * their device mapping (NVLink-C2C on GB300: coherent loads and stores from the SMs)
 * and puts the identity back, so the scratch is ready for the next call; the pixels
 * no line drew never cross the link.  max: host = std::max(host, max of the lines'
 * values), which is the sequential result (max is exact); sum: host + (sum of the
 * lines' values), the sum in another order. */
template <typename T> struct IdentityBits;
template <> struct IdentityBits<float> {
    using U = unsigned;
    static __host__ __device__ U max_bits() { return 0xff800000u; }   /* -inf */
    static __host__ __device__ U sum_bits() { return 0x80000000u; }   /* -0   */
};
template <> struct IdentityBits<double> {
    using U = unsigned long long;
    static __host__ __device__ U max_bits() { return 0xfff0000000000000ull; }
    static __host__ __device__ U sum_bits() { return 0x8000000000000000ull; }
};

template <typename T>
__global__ void __launch_bounds__(kThreads)
fill_identity_kernel(T *__restrict__ p, long long n, typename IdentityBits<T>::U bits)
{
    using U = typename IdentityBits<T>::U;
    U *q = reinterpret_cast<U *>(p);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        q[i] = bits;
}

/* the host frames travel over NVLink-C2C in 64-byte blocks, and a block written
 * whole costs about two thirds of one written in part (measured on GB300): the combine
 * reads and writes every block that holds a drawn pixel whole, its other pixels
 * unchanged */
constexpr int kHostBlock = 64;

template <typename T, int OV>
__device__ __forceinline__ void combine_pixel(T *host, typename IdentityBits<T>::U *sb,
                                              long long i, typename IdentityBits<T>::U id)
{
    const auto b = sb[i];
    if (b != id) {
        T d;
        memcpy(&d, &b, sizeof d);
        const T h = host[i];
        host[i] = OV == CBC_MAX ? (h < d ? d : h) : h + d;
        sb[i] = id;
    }
}

/* host[i] = combine(host[i], scratch[i]) where scratch holds a drawn value (not the
 * identity), and scratch back to the identity.  Pixels [head, head + n_units * E) form
 * whole 64-byte blocks of host memory (E pixels per 16-byte unit, 4 units per block, a
 * lane per unit); the head and the tail are done pixel by pixel.  A warp takes
 * kCombineRuns consecutive runs of 32 units (512 bytes) per step, one after another:
 * the link moved the frames faster in 1 KB runs than in 512-byte ones (measured on
 * GB300: 2.918 against 2.965 ms per detector-stack call), while spreading a block's
 * 64 bytes over one lane instead of four made every request scattered (6.83 ms). */
constexpr int kCombineRuns = 2;

template <typename T, int OV>
__global__ void __launch_bounds__(kThreads)
combine_host_kernel(T *__restrict__ host, T *__restrict__ scratch, long long n, long long head,
                    long long n_units, const DevStatus *st)
{
    using U = typename IdentityBits<T>::U;
    constexpr int E = 16 / (int)sizeof(T);
    if (st->flags & kFatal) return;          /* nothing was drawn */
    const U id = OV == CBC_MAX ? IdentityBits<T>::max_bits() : IdentityBits<T>::sum_bits();
    U *sb = reinterpret_cast<U *>(scratch);
    const int lane = threadIdx.x & 31;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    for (long long w0 = kCombineRuns * (tid - lane); w0 < n_units;
         w0 += kCombineRuns * nthreads) {
        for (int run = 0; run < kCombineRuns; run++) {
            const long long u = w0 + 32 * run + lane;
            const bool valid = u < n_units;   /* whole blocks: a lane group of 4 agrees */
            const long long i0 = head + u * E;
            U b[E];
            unsigned drawn = 0u;
            #pragma unroll
            for (int e = 0; e < E; e++) {
                b[e] = valid ? sb[i0 + e] : id;
                drawn |= (b[e] != id ? 1u : 0u) << e;
            }
            unsigned blk = drawn ? 1u : 0u;
            blk |= __shfl_xor_sync(0xffffffffu, blk, 1);
            blk |= __shfl_xor_sync(0xffffffffu, blk, 2);
            if (blk) {
                uint4 v = *reinterpret_cast<const uint4 *>(host + i0);
                T h[E];
                memcpy(h, &v, sizeof v);
                #pragma unroll
                for (int e = 0; e < E; e++) {
                    if ((drawn >> e) & 1u) {
                        T d;
                        memcpy(&d, &b[e], sizeof d);
                        h[e] = OV == CBC_MAX ? (h[e] < d ? d : h[e]) : h[e] + d;
                        sb[i0 + e] = id;
                    }
                }
                memcpy(&v, h, sizeof v);
                *reinterpret_cast<uint4 *>(host + i0) = v;
            }
        }
    }
    const long long body_end = head + n_units * E;
    const long long rest = head + (n - body_end);
    for (long long j = tid; j < rest; j += nthreads)
        combine_pixel<T, OV>(host, sb, j < head ? j : body_end + (j - head), id);
}

/* how the current device reaches host memory at `p`: page-locked memory through its
 * device mapping (CBC_HOST_MAPPED), pageable memory at its own address where the
 * device accesses pageable memory coherently through the host's page tables
 * (CBC_HOST_PAGEABLE), else not at all (CBC_HOST_NONE) */
int host_address(void *p, void **dev)
{
    *dev = nullptr;
    if (!p) return CBC_HOST_NONE;
    cudaPointerAttributes at{};
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return CBC_HOST_NONE;
    }
    if (at.type == cudaMemoryTypeHost) {
        void *m = nullptr;
        if (cudaHostGetDevicePointer(&m, p, 0) == cudaSuccess && m) {
            *dev = m;
            return CBC_HOST_MAPPED;
        }
        cudaGetLastError();
        return CBC_HOST_NONE;
    }
    if (at.type != cudaMemoryTypeUnregistered) return CBC_HOST_NONE;   /* device memory */
    int d = 0, pageable = 0, host_tables = 0;
    if (cudaGetDevice(&d) != cudaSuccess) {
        cudaGetLastError();
        return CBC_HOST_NONE;
    }
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, d);
    cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, d);
    if (!(pageable && host_tables)) return CBC_HOST_NONE;
    *dev = p;
    return CBC_HOST_PAGEABLE;
}

template <typename T>
int draw_lines_host_impl(T *host_out, long long n_frames, long long H, long long W,
                         const T *lines, long long n_lines, const void *idxs, int idx_bytes,
                         T max_val, int kernel, int overlap, T *scratch, int fill,
                         void *workspace, size_t ws_bytes, long long capacity,
                         long long ck_capacity, const cbc_tuning *tuning, void *stream)
{
    g_error.clear();
    const long long n = n_frames * H * W;
    if (n_frames < 0 || H < 0 || W < 0) return fail(CBC_ERR_INVALID, "negative size");
    if (overlap != CBC_SUM && overlap != CBC_MAX)
        return fail(CBC_ERR_INVALID, "Invalid overlap keyword");
    if (n > 0 && (!host_out || !scratch)) return fail(CBC_ERR_INVALID, "null pointer");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    T *dev_host = nullptr;
    if (n > 0) {
        void *p = nullptr;
        if (host_address(host_out, &p) == CBC_HOST_NONE)
            return fail(CBC_ERR_INVALID, "out is not host memory the device can address");
        dev_host = static_cast<T *>(p);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long most = (long long)(sms > 0 ? sms : 132) * 16;
    long long blocks = (n + kThreads - 1) / kThreads;
    if (blocks > most) blocks = most;
    using U = typename IdentityBits<T>::U;
    const U id = overlap == CBC_MAX ? IdentityBits<T>::max_bits() : IdentityBits<T>::sum_bits();
    if (fill && n > 0) {
        fill_identity_kernel<T><<<(unsigned)blocks, kThreads, 0, s>>>(scratch, n, id);
        note_launches(1);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    }
    int rc = draw_lines_impl<T>(scratch, n_frames, H, W, lines, n_lines, idxs, idx_bytes, max_val,
                                kernel, overlap, workspace, ws_bytes, capacity, ck_capacity,
                                tuning, stream);
    if (rc != CBC_OK) return rc;
    if (n > 0) {
        const DevStatus *st = reinterpret_cast<const DevStatus *>(workspace);
        /* whole 64-byte blocks from the first block boundary of the host frames on */
        const uintptr_t addr = reinterpret_cast<uintptr_t>(host_out);
        long long head = n, n_units = 0;
        if (addr % sizeof(T) == 0) {
            head = (long long)(((kHostBlock - addr % kHostBlock) % kHostBlock) / sizeof(T));
            if (head > n) head = n;
            const long long per_block = kHostBlock / (long long)sizeof(T);
            n_units = (n - head) / per_block * (kHostBlock / 16);
        }
        if (overlap == CBC_MAX)
            combine_host_kernel<T, CBC_MAX><<<(unsigned)blocks, kThreads, 0, s>>>(
                dev_host, scratch, n, head, n_units, st);
        else
            combine_host_kernel<T, CBC_SUM><<<(unsigned)blocks, kThreads, 0, s>>>(
                dev_host, scratch, n, head, n_units, st);
        note_launches(1);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    }
    return CBC_OK;
}

bool draw_workspace_parts(long long n_frames, long long H, long long W, long long n_lines,
                          long long capacity, long long ck_capacity, size_t elem,
                          const cbc_tuning *tuning, size_t *recs, size_t *cks)
{
    Resolved t;
    std::string why;
    if (!resolve_tuning(tuning, t, why)) return false;
    const Layout L = make_layout(n_frames, H, W, n_lines, capacity, ck_capacity,
                                 elem == 4 ? sizeof(LineRec<float>) : sizeof(LineRec<double>),
                                 elem == 4 ? sizeof(Checkpoint<float>) : sizeof(Checkpoint<double>),
                                 t);
    *recs = L.recs;
    *cks = L.cks;
    return true;
}

}  // namespace cbc

extern "C" {

int cbc_host_access(const void *host_ptr, int32_t *mode)
{
    cbc::clear_error();
    if (!mode) return cbc::fail(CBC_ERR_INVALID, "null mode pointer");
    void *dev_ptr = nullptr;
    *mode = cbc::host_address(const_cast<void *>(host_ptr), &dev_ptr);
    return CBC_OK;
}

int cbc_draw_lines_host_f32(float *host_out, int64_t n_frames, int64_t height, int64_t width,
                            const float *lines, int64_t n_lines, const void *idxs,
                            int32_t idx_bytes, float max_val, int32_t kernel, int32_t overlap,
                            float *scratch, int32_t fill, void *workspace,
                            size_t workspace_bytes, int64_t pair_capacity,
                            int64_t checkpoint_capacity, const cbc_tuning *tuning, void *stream)
{
    return cbc::draw_lines_host_impl<float>(host_out, n_frames, height, width, lines, n_lines,
                                            idxs, idx_bytes, max_val, kernel, overlap, scratch,
                                            fill, workspace, workspace_bytes, pair_capacity,
                                            checkpoint_capacity, tuning, stream);
}

int cbc_draw_lines_host_f64(double *host_out, int64_t n_frames, int64_t height, int64_t width,
                            const double *lines, int64_t n_lines, const void *idxs,
                            int32_t idx_bytes, double max_val, int32_t kernel, int32_t overlap,
                            double *scratch, int32_t fill, void *workspace,
                            size_t workspace_bytes, int64_t pair_capacity,
                            int64_t checkpoint_capacity, const cbc_tuning *tuning, void *stream)
{
    return cbc::draw_lines_host_impl<double>(host_out, n_frames, height, width, lines, n_lines,
                                             idxs, idx_bytes, max_val, kernel, overlap, scratch,
                                             fill, workspace, workspace_bytes, pair_capacity,
                                             checkpoint_capacity, tuning, stream);
}


size_t cbc_draw_lines_workspace_size(int64_t n_frames, int64_t height, int64_t width,
                                     int64_t n_lines, int64_t pair_capacity,
                                     int64_t checkpoint_capacity, int32_t elem_bytes,
                                     const cbc_tuning *tuning)
{
    cbc::Resolved t;
    std::string why;
    if (!cbc::resolve_tuning(tuning, t, why)) return 0;
    if (n_frames < 0 || height < 0 || width < 0 || n_lines < 0 || pair_capacity < 0 ||
        checkpoint_capacity < 0)
        return 0;
    size_t rec = elem_bytes == 8 ? sizeof(cbc::LineRec<double>) : sizeof(cbc::LineRec<float>);
    size_t ck = elem_bytes == 8 ? sizeof(cbc::Checkpoint<double>) : sizeof(cbc::Checkpoint<float>);
    return cbc::make_layout(n_frames, height, width, n_lines, pair_capacity, checkpoint_capacity,
                            rec, ck, t).total;
}

int cbc_draw_lines_f32(float *out, int64_t n_frames, int64_t height, int64_t width,
                       const float *lines, int64_t n_lines, const void *idxs, int32_t idx_bytes,
                       float max_val, int32_t kernel, int32_t overlap, void *workspace,
                       size_t workspace_bytes, int64_t pair_capacity,
                       int64_t checkpoint_capacity, const cbc_tuning *tuning, void *stream)
{
    return cbc::draw_lines_impl<float>(out, n_frames, height, width, lines, n_lines, idxs,
                                       idx_bytes, max_val, kernel, overlap, workspace,
                                       workspace_bytes, pair_capacity, checkpoint_capacity,
                                       tuning, stream);
}

int cbc_draw_lines_f64(double *out, int64_t n_frames, int64_t height, int64_t width,
                       const double *lines, int64_t n_lines, const void *idxs, int32_t idx_bytes,
                       double max_val, int32_t kernel, int32_t overlap, void *workspace,
                       size_t workspace_bytes, int64_t pair_capacity,
                       int64_t checkpoint_capacity, const cbc_tuning *tuning, void *stream)
{
    return cbc::draw_lines_impl<double>(out, n_frames, height, width, lines, n_lines, idxs,
                                        idx_bytes, max_val, kernel, overlap, workspace,
                                        workspace_bytes, pair_capacity, checkpoint_capacity,
                                        tuning, stream);
}

int cbc_draw_lines_csr_f32(float *out, int64_t n_frames, int64_t height, int64_t width,
                           const float *lines, int64_t n_lines, const int64_t *frame_offsets,
                           float max_val, int32_t kernel, int32_t overlap, void *workspace,
                           size_t workspace_bytes, int64_t pair_capacity,
                           int64_t checkpoint_capacity, const cbc_tuning *tuning, void *stream)
{
    if (!frame_offsets) return cbc::fail(CBC_ERR_INVALID, "null frame_offsets");
    return cbc::draw_lines_impl<float>(out, n_frames, height, width, lines, n_lines, nullptr, 0,
                                       max_val, kernel, overlap, workspace, workspace_bytes,
                                       pair_capacity, checkpoint_capacity, tuning, stream,
                                       frame_offsets);
}

int cbc_draw_lines_csr_f64(double *out, int64_t n_frames, int64_t height, int64_t width,
                           const double *lines, int64_t n_lines, const int64_t *frame_offsets,
                           double max_val, int32_t kernel, int32_t overlap, void *workspace,
                           size_t workspace_bytes, int64_t pair_capacity,
                           int64_t checkpoint_capacity, const cbc_tuning *tuning, void *stream)
{
    if (!frame_offsets) return cbc::fail(CBC_ERR_INVALID, "null frame_offsets");
    return cbc::draw_lines_impl<double>(out, n_frames, height, width, lines, n_lines, nullptr, 0,
                                        max_val, kernel, overlap, workspace, workspace_bytes,
                                        pair_capacity, checkpoint_capacity, tuning, stream,
                                        frame_offsets);
}

int cbc_draw_lines_max_winner_f32(float *out, int32_t *winner, uint64_t *packed,
                                  int64_t n_frames, int64_t height, int64_t width,
                                  const float *lines, int64_t n_lines, const void *idxs,
                                  int32_t idx_bytes, float max_val, int32_t kernel,
                                  void *workspace, size_t workspace_bytes, int64_t pair_capacity,
                                  int64_t checkpoint_capacity, void *stream)
{
    if (n_lines > 0 && n_frames * height * width > 0 && (!packed || (!out != !winner)))
        return cbc::fail(CBC_ERR_INVALID, "null packed, or only one of out and winner");
    cbc_tuning t{};
    t.strategy = CBC_STRATEGY_LINES;
    return cbc::draw_lines_impl<float>(out, n_frames, height, width, lines, n_lines, idxs,
                                       idx_bytes, max_val, kernel, CBC_MAX, workspace,
                                       workspace_bytes, pair_capacity, checkpoint_capacity, &t,
                                       stream, nullptr,
                                       reinterpret_cast<unsigned long long *>(packed), winner);
}

int cbc_read_status(const void *workspace, cbc_status *status, void *stream)
{
    cbc::g_error.clear();
    if (!workspace || !status) return cbc::fail(CBC_ERR_INVALID, "null pointer");
    /* a page-locked copy target per host thread (one small block, kept until exit)
     * makes the read a plain DMA; pageable memory is the fallback */
    static thread_local cbc::DevStatus *pinned = nullptr;
    static thread_local bool pinned_tried = false;
    if (!pinned_tried) {
        pinned_tried = true;
        if (cudaMallocHost(reinterpret_cast<void **>(&pinned), sizeof(cbc::DevStatus)) != cudaSuccess) {
            pinned = nullptr;
            cudaGetLastError();
        }
    }
    cbc::DevStatus local;
    cbc::DevStatus *dst = pinned ? pinned : &local;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(dst, workspace, sizeof *dst, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cbc::fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    const cbc::DevStatus d = *dst;
    status->flags = d.flags;
    status->strategy = d.strategy;
    status->bad_line = (int64_t)d.bad_line;
    status->idx_min = d.idx_min;
    status->idx_max = d.idx_max;
    status->pairs_needed = (int64_t)d.pairs;
    status->checkpoints_needed = (int64_t)d.cks;
    return CBC_OK;
}

size_t cbc_status_bytes(void) { return sizeof(cbc::DevStatus); }

int cbc_copy_status_async(const void *workspace, void *dst, void *stream)
{
    cbc::g_error.clear();
    if (!workspace || !dst) return cbc::fail(CBC_ERR_INVALID, "null pointer");
    cudaError_t e = cudaMemcpyAsync(dst, workspace, sizeof(cbc::DevStatus), cudaMemcpyDeviceToHost,
                                    static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cbc::fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    return CBC_OK;
}

int cbc_decode_status(const void *src, cbc_status *status)
{
    cbc::g_error.clear();
    if (!src || !status) return cbc::fail(CBC_ERR_INVALID, "null pointer");
    cbc::DevStatus d;
    std::memcpy(&d, src, sizeof d);
    status->flags = d.flags;
    status->strategy = d.strategy;
    status->bad_line = (int64_t)d.bad_line;
    status->idx_min = d.idx_min;
    status->idx_max = d.idx_max;
    status->pairs_needed = (int64_t)d.pairs;
    status->checkpoints_needed = (int64_t)d.cks;
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
        profile->launches = cbc::g_launches.load();
        profile->ms_prep = p.ms[0];
        profile->ms_offsets = p.ms[1];
        profile->ms_fill = p.ms[2];
        profile->ms_render = p.ms[3];
    }
    if (reset) {
        cbc::g_launches.store(0);
        p.calls = 0;
        for (double &m : p.ms) m = 0.0;
    }
    return CBC_OK;
}

const char *cbc_last_error(void) { return cbc::g_error.c_str(); }

const char *cbc_version(void) { return CBC_VERSION; }

}  // extern "C"

/* ---- no-allocation entry point ---------------------------------------------------
 * The lines-strategy kernels with their scratch (status block, line records, walk
 * checkpoints) in one fixed device array of this file instead of a caller workspace. */

namespace cbc {

constexpr size_t kNoallocRecOffset = 256;
static_assert(sizeof(DevStatus) <= kNoallocRecOffset, "the status block outgrew its slot");
constexpr size_t kNoallocCkOffset =
    kNoallocRecOffset + (sizeof(LineRec<float>) * CBC_NOALLOC_MAX_LINES + 255) / 256 * 256;
constexpr size_t kNoallocBytes =
    kNoallocCkOffset + sizeof(Checkpoint<float>) * CBC_NOALLOC_MAX_CHECKPOINTS;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

/* the array's address on the current device.  Looked up on every call: the address
 * belongs to the current context, and a context created after cudaDeviceReset may
 * place the array elsewhere, so a cached value could go stale. */
int noalloc_scratch(unsigned char **base)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
        return fail(CBC_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    *base = static_cast<unsigned char *>(p);
    return CBC_OK;
}

int draw_lines_noalloc(float *out, long long n_frames, long long H, long long W,
                       const float *lines, long long n_lines, const void *idxs, int idx_bytes,
                       float max_val, int kernel, int overlap, void *stream)
{
    g_error.clear();
    if (n_frames < 0 || H < 0 || W < 0 || n_lines < 0)
        return fail(CBC_ERR_INVALID, "negative size");
    if (H > INT_MAX / 2 || W > INT_MAX / 2)
        return fail(CBC_ERR_INVALID, "frame dimensions must be below 2^30");
    if (n_frames > INT_MAX)     /* line records hold the frame as a 32-bit index */
        return fail(CBC_ERR_INVALID, "n_frames must not exceed 2^31 - 1");
    if (kernel < 0 || kernel > 4) return fail(CBC_ERR_INVALID, "Invalid kernel type");
    if (overlap != CBC_SUM && overlap != CBC_MAX)
        return fail(CBC_ERR_INVALID, "Invalid overlap keyword");
    if (idxs && idx_bytes != 4 && idx_bytes != 8)
        return fail(CBC_ERR_INVALID, "idx_bytes must be 4 or 8");
    if (!idxs && n_lines > 0 && n_frames != 1 && n_frames != n_lines)
        return fail(CBC_ERR_INVALID, "idxs has an incompatible size (" + std::to_string(n_lines) +
                                         " != " + std::to_string(n_frames) + ")");
    if (n_lines > CBC_NOALLOC_MAX_LINES)
        return fail(CBC_ERR_INVALID, "n_lines " + std::to_string(n_lines) +
                                         " exceeds the no-allocation maximum of " +
                                         std::to_string(CBC_NOALLOC_MAX_LINES));
    if (n_lines > 0 && (!out || !lines) && n_frames * H * W > 0)
        return fail(CBC_ERR_INVALID, "null pointer");
    unsigned char *base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc != CBC_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DevStatus *st = reinterpret_cast<DevStatus *>(base);
    LineRec<float> *recs = reinterpret_cast<LineRec<float> *>(base + kNoallocRecOffset);
    Checkpoint<float> *cks = reinterpret_cast<Checkpoint<float> *>(base + kNoallocCkOffset);
    init_status_kernel<<<1, 1, 0, s>>>(st, CBC_STRATEGY_LINES);  /* a clean status per call */
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (n_lines > 0) {
        Geometry g;
        g.H = (int)H;
        g.W = (int)W;
        g.tile_w = g.tile_h = kDefaultTileW;
        g.tiles_x = g.tiles_y = 1;
        const unsigned nb = (unsigned)((n_lines + kThreads - 1) / kThreads);
        if (idxs && idx_bytes == 8)
            prep_kernel<float, int64_t, false, true><<<nb, kThreads, 0, s>>>(
                lines, idxs, n_lines, n_frames, g, recs, nullptr, cks,
                CBC_NOALLOC_MAX_CHECKPOINTS, st, nullptr);
        else
            prep_kernel<float, int32_t, false, true><<<nb, kThreads, 0, s>>>(
                lines, idxs, n_lines, n_frames, g, recs, nullptr, cks,
                CBC_NOALLOC_MAX_CHECKPOINTS, st, nullptr);
        note_launches(1);
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
        if (n_frames * H * W > 0) {
            SegArgs<float> sg;
            sg.out = out;
            sg.max_val = max_val;
            sg.d.recs = recs;
            sg.d.cks = cks;
            sg.d.H = (int)H;
            sg.d.W = (int)W;
            sg.d.st = st;
            sg.d.work = &st->work;
            e = launch_segments_k<float>(sg, kernel, overlap, s);
            if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
        }
    }
    DevStatus hs;
    e = cudaMemcpyAsync(&hs, st, sizeof hs, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (hs.flags & (1 << CBC_ERR_INDEX))
        return fail(CBC_ERR_INDEX, "idxs range (" + std::to_string(hs.idx_min) + ", " +
                                       std::to_string(hs.idx_max) + ") is outside of (0, " +
                                       std::to_string(n_frames) + ")");
    if (hs.flags & (1 << CBC_ERR_RANGE))
        return fail(CBC_ERR_RANGE, "line " + std::to_string(hs.bad_line) +
                                       ": its walk is longer than CBC_MAX_WALK pixels");
    if (hs.flags & (1 << CBC_ERR_CAPACITY))
        return fail(CBC_ERR_CAPACITY, "the walks need " + std::to_string(hs.cks) +
                                          " checkpoints, more than the no-allocation maximum of " +
                                          std::to_string(CBC_NOALLOC_MAX_CHECKPOINTS));
    return CBC_OK;
}

}  // namespace cbc

extern "C" int cbc_draw_lines_f32_noalloc(float *out, int64_t n_frames, int64_t height,
                                          int64_t width, const float *lines, int64_t n_lines,
                                          const void *idxs, int32_t idx_bytes, float max_val,
                                          int32_t kernel, int32_t overlap, void *stream)
{
    return cbc::draw_lines_noalloc(out, n_frames, height, width, lines, n_lines, idxs, idx_bytes,
                                   max_val, kernel, overlap, stream);
}
