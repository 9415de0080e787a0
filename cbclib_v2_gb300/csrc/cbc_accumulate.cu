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
 *   max, sum  a term's value at a pixel must be complete before it is added: per
 *   sum, max  (term, pixel) values go into an open-addressing hash table in the
 *             workspace (key term << 32 | pixel, linear probing, at most 64 probes),
 *             combined there with atomics, then one pass over the table merges every
 *             entry into `out`.  A full table sets CBC_ERR_CAPACITY and the call draws
 *             nothing; pairs_needed then holds a table capacity to retry with.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <limits.h>
#include <string>

#include "cbc_accumulate.cuh"

namespace cbc {

template <typename T, int K, int MODE>
struct AccumAct {
    static constexpr bool kNeedsGeometry = false;
    static constexpr bool kNeedsError = true;
    T *out;
    T max_val;
    int W;
    const float *gtab;
    const int *term_of_line;
    unsigned long long *keys;
    T *vals;
    unsigned long long mask;       /* table capacity - 1 (a power of two) */
    DevStatus *st;
    struct Pre {};
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
    act.st = a.d.st;
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
    if (table && (table_capacity < 1 || (table_capacity & (table_capacity - 1))))
        return fail(CBC_ERR_INVALID, "table_capacity must be a power of two");
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
    if (e == cudaSuccess && table) e = clear_table(keys, vals, table_capacity, s);
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
    a.mask = table ? (unsigned long long)table_capacity - 1ull : 0ull;
    switch (kernel) {
    case CBC_BIWEIGHT:    e = launch_accumulate<T, CBC_BIWEIGHT>(a, mode, s); break;
    case CBC_GAUSSIAN:    e = launch_accumulate<T, CBC_GAUSSIAN>(a, mode, s); break;
    case CBC_PARABOLIC:   e = launch_accumulate<T, CBC_PARABOLIC>(a, mode, s); break;
    case CBC_RECTANGULAR: e = launch_accumulate<T, CBC_RECTANGULAR>(a, mode, s); break;
    default:              e = launch_accumulate<T, CBC_TRIANGULAR>(a, mode, s); break;
    }
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (table) {
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
