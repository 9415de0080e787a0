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
 * The pixels are exactly the forward's: drive_segments (cbc_common.cuh) enumerates the
 * walk with the reference's arithmetic.  For max overlap a first pass records, per
 * pixel, the smallest line index whose exact value equals the final pixel value (and
 * exceeds the value before drawing): sequential std::max keeps the first such line,
 * so only that line receives the pixel's gradient.  Per-line sums are accumulated per
 * segment in shared memory, then in double in global memory.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <limits.h>
#include <string>

#include "cbc_common.cuh"

namespace cbc {


/* max overlap: winner[p] = min over lines l with v_l(p) == image[p] > out0[p] */
template <typename T, int K>
struct WinnerAct {
    static constexpr bool kNeedsGeometry = false;
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
    __device__ __forceinline__ void item_begin(int) {}
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

template <typename T, int K>
__device__ __forceinline__ T kappa_of(T d, T w, T max_val)
{
    const T x = d / w, ww = w * w;
    switch (K) {
    case CBC_BIWEIGHT:  return max_val * T(-3.75) * (T(1) - x * x) / ww;
    case CBC_GAUSSIAN:  return max_val * T(-9) * T(CBC_GAUSS_C) * exp(T(-4.5) * x * x) / ww;
    case CBC_PARABOLIC: return max_val * T(-1.5) / ww;
    case CBC_RECTANGULAR: return T(0);
    default:            return d > T(0) ? -max_val / (d * w) : T(0);
    }
}

template <typename T, int K, int OV>
struct BackwardAct {
    static constexpr bool kNeedsGeometry = true;
    /* max overlap: a pixel whose winner is this line was drawn by it, so the error is
     * not needed; sum overlap: every drawn pixel (error <= 1) */
    static constexpr bool kNeedsError = OV != CBC_MAX;
    const T *grad_out;   /* dL/dI, or NULL with image and target: L = sum((I - T)^2) */
    const T *image;
    const T *target;
    const unsigned long long *packed;   /* max overlap: (value bits, ~winner) per pixel */
    const int *winner;   /* max overlap */
    double *gacc;        /* (N, 5) */
    T (*acc)[5];         /* this warp's per-slot accumulators (shared memory) */
    T max_val;
    int W;
    __device__ __forceinline__ void item_begin(int lane) {
        #pragma unroll
        for (int k = 0; k < 5; k++) acc[lane][k] = T(0);
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
    /* max overlap: the winner first, the gradient only for the winning line; sum: the
     * gradient of every pixel */
    struct Pre {
        int win;
        T g;
    };
    __device__ __forceinline__ T grad_at(long long at) const {
        return grad_out ? grad_out[at] : T(2) * (image[at] - target[at]);
    }
    __device__ __forceinline__ Pre prefetch(const SlotTable<T> &S, int slot, int px, int py) const {
        const long long at = S.fbase[slot] + (long long)py * W + px;
        Pre p;
        if (OV == CBC_MAX && packed) {
            /* value and winner in one load, the target beside it: the squared-loss
             * gradient of the winning line needs no second round trip */
            const unsigned long long k = packed[at];
            const unsigned hi = (unsigned)(k >> 32);
            p.win = hi ? (int)(0xffffffffu - (unsigned)k) : 0x7f7f7f7f;
            p.g = target ? T(2) * ((T)__uint_as_float(hi) - target[at]) : T(0);
        } else {
            p.win = OV == CBC_MAX ? winner[at] : 0;
            p.g = OV == CBC_MAX ? T(0) : grad_at(at);
        }
        return p;
    }
    __device__ __forceinline__ void pixel(const SlotTable<T> &S, int slot, int px, int py, T, T,
                                          T, const Pre &p) {
        if (OV == CBC_MAX && p.win != S.line[slot]) return;
        const T g = (OV == CBC_MAX && !(packed && target))
                        ? grad_at(S.fbase[slot] + (long long)py * W + px) : p.g;
        if (g == T(0)) return;
        const T x0 = S.x0[slot], y0 = S.y0[slot], t0 = S.t0[slot], t1 = S.t1[slot];
        const T w = S.w[slot];
        const T X = (T)px, Y = (T)py;
        const T cx = x0 + T(0.5) * t0, cy = y0 + T(0.5) * t1;
        const T mag = t0 * t0 + t1 * t1;
        T t = ((X - cx) * t0 + (Y - cy) * t1) / mag;
        t = t < T(-0.5) ? T(-0.5) : (t > T(0.5) ? T(0.5) : t);
        const T dx = cx + t * t0 - X, dy = cy + t * t1 - Y;
        const T d2 = dx * dx + dy * dy;
        const T d = sqrt(d2);
        const T G = g * kappa_of<T, K>(d, w, max_val);
        if (G == T(0)) return;
        const T s = t + T(0.5);
        atomicAdd(&acc[slot][0], G * (T(1) - s) * dx);
        atomicAdd(&acc[slot][1], G * (T(1) - s) * dy);
        atomicAdd(&acc[slot][2], G * s * dx);
        atomicAdd(&acc[slot][3], G * s * dy);
        atomicAdd(&acc[slot][4], -G * d2 / w);
    }
};

template <typename T>
struct AdjArgs {
    DriveArgs<T> d;
    const T *grad_out;
    const T *image;
    const T *out0;
    const T *target;
    const unsigned long long *packed;
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

template <typename T, int K, int OV>
__global__ void __launch_bounds__(kSegWarps * 32)
backward_kernel(AdjArgs<T> a)
{
    __shared__ T acc_s[kSegWarps][32][5];
    BackwardAct<T, K, OV> act;
    act.grad_out = a.grad_out;
    act.image = a.image;
    act.target = a.target;
    act.packed = a.packed;
    act.winner = a.winner;
    act.gacc = a.gacc;
    act.acc = acc_s[threadIdx.x >> 5];
    act.max_val = a.max_val;
    act.W = a.d.W;
    drive_segments(a.d, act);
}

template <typename T>
__global__ void finalize_kernel(const double *gacc, T *grad_lines, long long n)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) grad_lines[i] = (T)gacc[i];
}

struct AdjLayout {
    size_t status, recs, cks, gacc, total;
};

AdjLayout adj_layout(long long n_lines, long long ck_capacity, size_t rec_bytes, size_t ck_bytes)
{
    auto up = [](size_t v) { return (v + 255) / 256 * 256; };
    AdjLayout L;
    size_t off = 0;
    L.status = off; off = up(off + sizeof(DevStatus));
    L.recs = off;   off = up(off + rec_bytes * (size_t)n_lines);
    L.cks = off;    off = up(off + ck_bytes * (size_t)ck_capacity);
    L.gacc = off;   off = up(off + sizeof(double) * 5 * (size_t)n_lines);
    L.total = off;
    return L;
}

template <typename T, int K>
cudaError_t launch_adjoint(const AdjArgs<T> &aa, int overlap, bool winner_known, cudaStream_t s)
{
    if (overlap == CBC_MAX) {
        if (!winner_known) {
            const unsigned grid = resident_grid(winner_kernel<T, K>, kSegWarps * 32);
            winner_kernel<T, K><<<grid, kSegWarps * 32, 0, s>>>(aa);
            note_launches(1);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
            e = cudaMemsetAsync(aa.d.work, 0, sizeof(unsigned long long), s);
            if (e != cudaSuccess) return e;
        }
        backward_kernel<T, K, CBC_MAX><<<resident_grid(backward_kernel<T, K, CBC_MAX>,
                                                       kSegWarps * 32),
                                         kSegWarps * 32, 0, s>>>(aa);
    } else {
        backward_kernel<T, K, CBC_SUM><<<resident_grid(backward_kernel<T, K, CBC_SUM>,
                                                       kSegWarps * 32),
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
    if (packed && (overlap != CBC_MAX || sizeof(T) != sizeof(float)))
        return fail(CBC_ERR_INVALID, "packed winners are for float32 max overlap");
    AdjLayout L = adj_layout(n_lines, ck_capacity, sizeof(LineRec<T>), sizeof(Checkpoint<T>));
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
    e = cudaMemsetAsync(gacc, 0, sizeof(double) * 5 * (size_t)n_lines, s);
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    Geometry g;
    g.H = (int)H;
    g.W = (int)W;
    g.tile_w = g.tile_h = 64;
    g.tiles_x = g.tiles_y = 1;
    const unsigned nb = (unsigned)((n_lines + 255) / 256);
    if (idxs && idx_bytes == 8)
        prep_kernel<T, int64_t, false, true><<<nb, 256, 0, s>>>(lines, idxs, n_lines, n_frames, g,
                                                                recs, nullptr, cks, ck_capacity, st,
                                                                nullptr);
    else
        prep_kernel<T, int32_t, false, true><<<nb, 256, 0, s>>>(lines, idxs, n_lines, n_frames, g,
                                                                recs, nullptr, cks, ck_capacity, st,
                                                                nullptr);
    note_launches(1);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    if (pixels) {
        if (overlap == CBC_MAX && !winner_known) {
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
        aa.grad_out = grad_out;
        aa.image = image;
        aa.out0 = out0;
        aa.target = target;
        aa.packed = packed;
        aa.winner = winner;
        aa.gacc = gacc;
        aa.max_val = max_val;
        switch (kernel) {
        case CBC_BIWEIGHT:    e = launch_adjoint<T, CBC_BIWEIGHT>(aa, overlap, winner_known, s); break;
        case CBC_GAUSSIAN:    e = launch_adjoint<T, CBC_GAUSSIAN>(aa, overlap, winner_known, s); break;
        case CBC_PARABOLIC:   e = launch_adjoint<T, CBC_PARABOLIC>(aa, overlap, winner_known, s); break;
        case CBC_RECTANGULAR: e = launch_adjoint<T, CBC_RECTANGULAR>(aa, overlap, winner_known, s); break;
        default:              e = launch_adjoint<T, CBC_TRIANGULAR>(aa, overlap, winner_known, s); break;
        }
        if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    }
    const long long n5 = 5 * n_lines;
    finalize_kernel<T><<<(unsigned)((n5 + 255) / 256), 256, 0, s>>>(gacc, grad_lines, n5);
    note_launches(1);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CBC_ERR_CUDA, cudaGetErrorString(e));
    return CBC_OK;
}

}  // namespace cbc

extern "C" {

size_t cbc_draw_lines_backward_workspace_size(int64_t n_lines, int64_t checkpoint_capacity,
                                              int32_t elem_bytes)
{
    if (n_lines < 0 || checkpoint_capacity < 0) return 0;
    size_t rec = elem_bytes == 8 ? sizeof(cbc::LineRec<double>) : sizeof(cbc::LineRec<float>);
    size_t ck = elem_bytes == 8 ? sizeof(cbc::Checkpoint<double>) : sizeof(cbc::Checkpoint<float>);
    return cbc::adj_layout(n_lines, checkpoint_capacity, rec, ck).total;
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

}  // extern "C"
