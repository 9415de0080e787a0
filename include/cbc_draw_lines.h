/*
 * cbc_draw_lines.h — C ABI of the GB300 (sm_103a) streak-model rasteriser.
 *
 * Every entry point takes plain pointers and sizes; device pointers are CUDA device
 * memory of the current device, `stream` is a cudaStream_t (NULL = legacy default
 * stream).  Calls are stream-ordered and never synchronise the host, except
 * cbc_read_status(), which waits for the stream.  No C++ exception crosses the ABI.
 *
 * Reference interfaces replaced (paths inside the cbclib_v2 project):
 *   bresenham.draw_lines           cbclib_v2/_src/src/bresenham.cpp:313-331 (pybind11,
 *                                   overloads <double,long> and <float,int>)
 *   cuda_draw_lines.draw_lines     cbclib_v2/_src/src/cuda_draw_lines.cu:1098-1113
 *   cuda_draw_lines.accumulate_lines  cbclib_v2/_src/src/cuda_draw_lines.cu:1076-1097
 * as called by cbclib_v2/_src/functions.py:235-254 (_draw_lines_cpu/_gpu) and
 * :151-173 (_accumulate_lines_cpu/_gpu).
 */
#ifndef CBC_DRAW_LINES_H
#define CBC_DRAW_LINES_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define CBC_API __attribute__((visibility("default")))
#else
#define CBC_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (host return values and device status flags) ------------------ */
#define CBC_OK              0
#define CBC_ERR_INVALID     1   /* bad argument: ValueError in the reference           */
#define CBC_ERR_INDEX       2   /* frame index out of range: IndexError (bresenham.cpp:32-34) */
#define CBC_ERR_CAPACITY    3   /* pair buffer too small; nothing was drawn, retry      */
#define CBC_ERR_CUDA        4   /* CUDA runtime error: RuntimeError (cupy_array.hpp:18-24);
                                   as a status flag: a device-side wait for an
                                   asynchronous copy gave up (the result is incomplete) */
#define CBC_ERR_RANGE       5   /* a line's walk is longer than CBC_MAX_WALK pixels     */
#define CBC_ERR_TERM        6   /* accumulate_lines: a term index out of range: IndexError
                                   (bresenham.cpp:182-188); status flag only          */

#define CBC_MAX_WALK (1 << 22)

/* profile kernels, enum order of kernels::type (include.hpp:470-479) */
#define CBC_BIWEIGHT    0
#define CBC_GAUSSIAN    1
#define CBC_PARABOLIC   2
#define CBC_RECTANGULAR 3
#define CBC_TRIANGULAR  4

/* overlap modes (bresenham.cpp:142-149: "sum" -> 0, "max" -> 1) */
#define CBC_SUM 0
#define CBC_MAX 1

/* render strategies */
#define CBC_STRATEGY_AUTO  0   /* the library's choice: the lines strategy            */
#define CBC_STRATEGY_TILES 1   /* (frame, tile) bins, shared-memory tiles, one pass out */
#define CBC_STRATEGY_LINES 2   /* warps of 32 lines, L2 reductions into out             */

/* render configuration; zeros select the built-in defaults */
typedef struct cbc_tuning {
    int32_t tile_w;        /* tile width in pixels (x), multiple of 4, 16..256        */
    int32_t tile_h;        /* tile height in pixels (y), 4..256                       */
    int32_t chunk_lines;   /* lines staged per shared-memory chunk, 1..32             */
    int32_t threads;       /* threads per render CTA: 128 or 256                      */
    int32_t strategy;      /* CBC_STRATEGY_*                                          */
    int32_t reserved;
} cbc_tuning;

/* device-side status, the first bytes of the workspace, read by cbc_read_status */
typedef struct cbc_status {
    int32_t flags;         /* bit (1 << CBC_ERR_x) for every error seen               */
    int32_t strategy;      /* CBC_STRATEGY_TILES or _LINES: the render the call ran   */
    int64_t bad_line;      /* smallest offending line index (INT64_MAX if none)       */
    int64_t idx_min;       /* smallest frame index in idxs (INT64_MAX if none)        */
    int64_t idx_max;       /* largest frame index in idxs (INT64_MIN if none)         */
    int64_t pairs_needed;  /* (line, tile) pairs the call produced                    */
    int64_t checkpoints_needed; /* walk checkpoints the call produced                 */
} cbc_status;

/* Bytes of device workspace a call with these sizes needs.  `pair_capacity` bounds
 * the (line, tile) pairs and `checkpoint_capacity` the walk checkpoints (one per 16
 * columns of each line's walk inside its frame); when a call produces more of
 * either, it draws nothing, sets CBC_ERR_CAPACITY and reports both counts, so the
 * caller can grow the workspace and repeat the call. */
CBC_API size_t cbc_draw_lines_workspace_size(int64_t n_frames, int64_t height, int64_t width,
                                             int64_t n_lines, int64_t pair_capacity,
                                             int64_t checkpoint_capacity, int32_t elem_bytes,
                                             const cbc_tuning *tuning);

/* draw_lines: out[(f, y, x)] = out ⊕ max_val·K(d/w) for every pixel the reference's
 * Bresenham walk of each line visits with error <= 1, ⊕ = + (CBC_SUM) or max (CBC_MAX).
 *   out    (n_frames, height, width) C-contiguous, updated in place
 *   lines  (n_lines, 5) C-contiguous rows x0, y0, x1, y1, width (xy order)
 *   idxs   (n_lines,) frame of each line, int32 (idx_bytes = 4) or int64 (8);
 *          NULL: frame 0 when n_frames == 1, frame i when n_frames == n_lines
 *          (bresenham.cpp:5-20), otherwise CBC_ERR_INVALID.
 * Returns CBC_OK or a host-detected error; device-detected errors (frame index out
 * of range, capacity, walk range) are left in the workspace status and leave `out`
 * untouched. */
CBC_API int cbc_draw_lines_f32(float *out, int64_t n_frames, int64_t height, int64_t width,
                               const float *lines, int64_t n_lines, const void *idxs,
                               int32_t idx_bytes, float max_val, int32_t kernel,
                               int32_t overlap, void *workspace, size_t workspace_bytes,
                               int64_t pair_capacity, int64_t checkpoint_capacity,
                               const cbc_tuning *tuning, void *stream);

CBC_API int cbc_draw_lines_f64(double *out, int64_t n_frames, int64_t height, int64_t width,
                               const double *lines, int64_t n_lines, const void *idxs,
                               int32_t idx_bytes, double max_val, int32_t kernel,
                               int32_t overlap, void *workspace, size_t workspace_bytes,
                               int64_t pair_capacity, int64_t checkpoint_capacity,
                               const cbc_tuning *tuning, void *stream);

/* Ragged stacks: the lines are grouped by frame and frame f owns lines
 * [frame_offsets[f], frame_offsets[f + 1]) (int64 CSR offsets, n_frames + 1 entries,
 * frame_offsets[0] == 0, frame_offsets[n_frames] == n_lines).  Otherwise as
 * cbc_draw_lines_f32 / _f64; offsets that break those rules are a device-detected
 * CBC_ERR_INDEX.  The call launches a fixed sequence of kernels and memsets and reads
 * nothing back, so it can be captured into a CUDA graph and replayed. */
CBC_API int cbc_draw_lines_csr_f32(float *out, int64_t n_frames, int64_t height, int64_t width,
                                   const float *lines, int64_t n_lines,
                                   const int64_t *frame_offsets, float max_val, int32_t kernel,
                                   int32_t overlap, void *workspace, size_t workspace_bytes,
                                   int64_t pair_capacity, int64_t checkpoint_capacity,
                                   const cbc_tuning *tuning, void *stream);

CBC_API int cbc_draw_lines_csr_f64(double *out, int64_t n_frames, int64_t height, int64_t width,
                                   const double *lines, int64_t n_lines,
                                   const int64_t *frame_offsets, double max_val, int32_t kernel,
                                   int32_t overlap, void *workspace, size_t workspace_bytes,
                                   int64_t pair_capacity, int64_t checkpoint_capacity,
                                   const cbc_tuning *tuning, void *stream);

/* Limits of cbc_draw_lines_f32_noalloc. */
#define CBC_NOALLOC_MAX_LINES       16384
#define CBC_NOALLOC_MAX_CHECKPOINTS 262144

/* cbc_draw_lines_f32 without any device allocation by the caller (no counterpart in
 * the reference, whose GPU path allocates on every call).
 *
 * Some callers cannot hand this library a workspace: a detector acquisition loop
 * that reserves its whole device memory budget before a run and must not stall on
 * cudaMalloc's implicit device synchronisation or fail half-way through a run when
 * memory is short, or a plugin hosted by a framework whose pool allocator owns every
 * byte of the device.  This entry point needs no memory from them: its scratch is one
 * fixed array inside the library, about 7.9 MB, held on every GPU that loads the
 * library until the process exits.
 *
 * Arguments and results are those of cbc_draw_lines_f32 (float32 only), with these
 * limits: n_lines <= CBC_NOALLOC_MAX_LINES, else CBC_ERR_INVALID before any work; and
 * the lines' walks inside their frames may need at most CBC_NOALLOC_MAX_CHECKPOINTS
 * checkpoints (one per 16 columns of each walk), else the call draws nothing and
 * returns CBC_ERR_CAPACITY; n_frames must not exceed 2^31 - 1 (else CBC_ERR_INVALID).
 * Every call looks up the array's device address for the current device and
 * context (cudaGetSymbolAddress), so the address is never reused across contexts,
 * e.g. after cudaDeviceReset.  The call synchronises `stream` (it reads the device
 * status back) and returns the call's full status (CBC_OK, CBC_ERR_INDEX,
 * CBC_ERR_CAPACITY, CBC_ERR_RANGE, ...; message in cbc_last_error).  All calls share
 * the one array and every call re-initialises it, so calls that overlap on the GPU
 * (unordered streams, or threads without ordering) race: issue them one after
 * another. */
CBC_API int cbc_draw_lines_f32_noalloc(float *out, int64_t n_frames, int64_t height,
                                       int64_t width, const float *lines, int64_t n_lines,
                                       const void *idxs, int32_t idx_bytes, float max_val,
                                       int32_t kernel, int32_t overlap, void *stream);

/* ---- adjoint (no counterpart in the reference) ----------------------------------
 * Gradient of draw_lines with respect to the line parameters, from the gradient of
 * the frames: grad_lines[i] = sum over the pixels p line i draws of
 * grad_out[p] * d(max_val K(d(p)/w))/d(x0, y0, x1, y1, w), over exactly the pixels the
 * forward draws.  For max overlap only the line whose value a pixel kept receives
 * that pixel's gradient: pass the forward's result `image`, the frames before drawing
 * `out0` (NULL: zeros) and a (n_frames, height, width) int32 `winner` buffer, which
 * comes back holding each pixel's winning line (0x7f7f7f7f where none drew the value).
 * `grad_lines` (n_lines, 5) is overwritten.  Device-detected errors are reported
 * through the workspace status as for cbc_draw_lines_*; capacity and walk limits as
 * there. */
CBC_API size_t cbc_draw_lines_backward_workspace_size(int64_t n_lines,
                                                      int64_t checkpoint_capacity,
                                                      int32_t elem_bytes);

CBC_API int cbc_draw_lines_backward_f32(const float *grad_out, int64_t n_frames,
                                        int64_t height, int64_t width, const float *lines,
                                        int64_t n_lines, const void *idxs, int32_t idx_bytes,
                                        float max_val, int32_t kernel, int32_t overlap,
                                        const float *image, const float *out0,
                                        int32_t *winner, float *grad_lines, void *workspace,
                                        size_t workspace_bytes, int64_t checkpoint_capacity,
                                        void *stream);

CBC_API int cbc_draw_lines_backward_f64(const double *grad_out, int64_t n_frames,
                                        int64_t height, int64_t width, const double *lines,
                                        int64_t n_lines, const void *idxs, int32_t idx_bytes,
                                        double max_val, int32_t kernel, int32_t overlap,
                                        const double *image, const double *out0,
                                        int32_t *winner, double *grad_lines, void *workspace,
                                        size_t workspace_bytes, int64_t checkpoint_capacity,
                                        void *stream);

/* Gradient of the squared loss L = sum((image - target)^2) with respect to the line
 * parameters, where image = out0 + draw_lines(lines) is the forward result (out0 NULL:
 * zeros).  Same as cbc_draw_lines_backward_* with grad_out = 2 (image - target), which
 * is formed per drawn pixel instead of being stored: the fused render -> loss ->
 * adjoint step of a streak fit.  No counterpart in the reference (new). */
CBC_API int cbc_squared_loss_backward_f32(const float *image, const float *target,
                                          int64_t n_frames, int64_t height, int64_t width,
                                          const float *lines, int64_t n_lines, const void *idxs,
                                          int32_t idx_bytes, float max_val, int32_t kernel,
                                          int32_t overlap, const float *out0, int32_t *winner,
                                          float *grad_lines, void *workspace,
                                          size_t workspace_bytes, int64_t checkpoint_capacity,
                                          void *stream);

CBC_API int cbc_squared_loss_backward_f64(const double *image, const double *target,
                                          int64_t n_frames, int64_t height, int64_t width,
                                          const double *lines, int64_t n_lines,
                                          const void *idxs, int32_t idx_bytes, double max_val,
                                          int32_t kernel, int32_t overlap, const double *out0,
                                          int32_t *winner, double *grad_lines, void *workspace,
                                          size_t workspace_bytes, int64_t checkpoint_capacity,
                                          void *stream);

/* The forward for max overlap into frames that start at zero, recording each pixel's
 * winner (the line sequential std::max keeps: the smallest index among the lines whose
 * value equals the pixel; 0x7f7f7f7f where no line raised the pixel above zero).
 * out (overwritten, no need to clear), winner: n_frames * height * width each;
 * packed: the same number of uint64 values that must be zero on entry and are zero
 * again on return.  With out = winner = NULL the call leaves packed holding, per
 * pixel, (value bits << 32) | (0xffffffff - winner) (0 where no line raised the pixel)
 * for cbc_draw_lines_backward_ex_f32, and the caller clears it before the next call.
 * Other arguments as cbc_draw_lines_f32 (lines strategy).  With
 * cbc_draw_lines_backward_ex_* (winner_known = 1, or packed) the adjoint skips its
 * winner pass.
 * No counterpart in the reference (new). */
CBC_API int cbc_draw_lines_max_winner_f32(float *out, int32_t *winner, uint64_t *packed,
                                          int64_t n_frames, int64_t height, int64_t width,
                                          const float *lines, int64_t n_lines, const void *idxs,
                                          int32_t idx_bytes, float max_val, int32_t kernel,
                                          void *workspace, size_t workspace_bytes,
                                          int64_t pair_capacity, int64_t checkpoint_capacity,
                                          void *stream);

/* cbc_draw_lines_backward_* generalised: grad_out NULL takes the squared loss
 * sum((image - target)^2) (as cbc_squared_loss_backward_*); winner_known = 1 uses
 * `winner` as filled by cbc_draw_lines_max_winner_f32 instead of recomputing it (max
 * overlap, frames that started at zero); packed (float32 max overlap) takes image and
 * winners from the pairs cbc_draw_lines_max_winner_f32 left with out = winner = NULL.
 * No counterpart in the reference (new). */
CBC_API int cbc_draw_lines_backward_ex_f32(const float *grad_out, const float *target,
                                           int64_t n_frames, int64_t height, int64_t width,
                                           const float *lines, int64_t n_lines,
                                           const void *idxs, int32_t idx_bytes, float max_val,
                                           int32_t kernel, int32_t overlap, const float *image,
                                           const float *out0, int32_t *winner,
                                           int32_t winner_known, const uint64_t *packed,
                                           float *grad_lines, void *workspace,
                                           size_t workspace_bytes, int64_t checkpoint_capacity,
                                           void *stream);

CBC_API int cbc_draw_lines_backward_ex_f64(const double *grad_out, const double *target,
                                           int64_t n_frames, int64_t height, int64_t width,
                                           const double *lines, int64_t n_lines,
                                           const void *idxs, int32_t idx_bytes, double max_val,
                                           int32_t kernel, int32_t overlap, const double *image,
                                           const double *out0, int32_t *winner,
                                           int32_t winner_known, const uint64_t *packed,
                                           double *grad_lines, void *workspace,
                                           size_t workspace_bytes, int64_t checkpoint_capacity,
                                           void *stream);

/* One step of a float32 max-overlap least-squares streak fit in one call: the forward
 * (cbc_draw_lines_max_winner_f32 into `packed`, no frames written), then the gradient
 * of L = sum((draw(lines) - target)^2) with respect to the (N, 5) lines into
 * grad_lines, in one pass over the packed words and the target that also zeroes
 * `packed` for the next call.  `packed` holds n_frames * height * width zeroed
 * uint64 on entry and is zero again on return.  loss_delta (device, may be NULL)
 * receives sum over drawn pixels of I (I - 2 target), i.e. L - sum(target^2).
 * The workspace (cbc_squared_loss_step_workspace_size) starts with the forward's, so
 * cbc_read_status on it reports the forward's errors and capacity needs.
 * No counterpart in the reference (new). */
CBC_API size_t cbc_squared_loss_step_workspace_size(int64_t n_frames, int64_t height,
                                                    int64_t width, int64_t n_lines,
                                                    int64_t pair_capacity,
                                                    int64_t checkpoint_capacity);

CBC_API int cbc_squared_loss_step_f32(const float *target, int64_t n_frames, int64_t height,
                                      int64_t width, const float *lines, int64_t n_lines,
                                      const void *idxs, int32_t idx_bytes, float max_val,
                                      int32_t kernel, uint64_t *packed, float *grad_lines,
                                      double *loss_delta, void *workspace,
                                      size_t workspace_bytes, int64_t pair_capacity,
                                      int64_t checkpoint_capacity, void *stream);

/* The same step for float32 sum overlap: `image` (n_frames * height * width device
 * floats) is zeroed and receives draw(lines); the adjoint then walks the forward's own
 * line records and walk checkpoints (no second preparation) and writes the gradient of
 * L = sum((image - target)^2) into grad_lines.  loss (device double, may be NULL)
 * receives L.  Workspace size: cbc_squared_loss_step_workspace_size; its start is the
 * forward's, so cbc_read_status on it reports the forward's errors and capacity
 * needs.  No counterpart in the reference (new). */
CBC_API int cbc_squared_loss_step_sum_f32(const float *target, float *image, int64_t n_frames,
                                          int64_t height, int64_t width, const float *lines,
                                          int64_t n_lines, const void *idxs, int32_t idx_bytes,
                                          float max_val, int32_t kernel, float *grad_lines,
                                          double *loss, void *workspace,
                                          size_t workspace_bytes, int64_t pair_capacity,
                                          int64_t checkpoint_capacity, void *stream);

/* How the current device reaches the host memory at host_ptr: CBC_HOST_MAPPED
 * (page-locked, through its device mapping), CBC_HOST_PAGEABLE (pageable memory,
 * coherently through the host's page tables) or CBC_HOST_NONE (not at all: the
 * frames must be copied).  No counterpart in the reference, whose host arrays are
 * always drawn on the CPU. */
#define CBC_HOST_NONE     0
#define CBC_HOST_MAPPED   1
#define CBC_HOST_PAGEABLE 2
CBC_API int cbc_host_access(const void *host_ptr, int32_t *mode);

/* draw_lines into frames in host memory that the kernels address directly over
 * NVLink-C2C on GB300: page-locked memory (cudaHostAlloc, or registered) through its
 * device mapping, or pageable memory (malloc, NumPy arrays) where the device reads
 * and writes it coherently through the host's page tables
 * (cudaDevAttrPageableMemoryAccess and cudaDevAttrPageableMemoryAccessUsesHostPageTables
 * both set); host_out must be writable.  The lines are drawn into
 * `scratch` (n_frames * height * width device elements), which must hold the
 * overlap's identity on entry (-inf for CBC_MAX, -0.0 for CBC_SUM) unless `fill` is 1
 * (the call writes it first); then the pixels some line drew are combined into
 * host_out and `scratch` gets the identity back.  Only drawn pixels cross the link.
 * lines and idxs are device arrays or host memory the device reads (cbc_host_access:
 * the kernels read each line and index once); other arguments, the workspace and the
 * errors as
 * cbc_draw_lines_f32 (an error leaves host_out untouched).  Host memory the device
 * cannot address (pageable memory on other systems) is rejected with CBC_ERR_INVALID
 * before anything runs.  Replaces the host-array path of the reference's
 * draw_lines (_src/functions.py:275-302, bresenham.cpp:313-331).  */
CBC_API int cbc_draw_lines_host_f32(float *host_out, int64_t n_frames, int64_t height,
                                    int64_t width, const float *lines, int64_t n_lines,
                                    const void *idxs, int32_t idx_bytes, float max_val,
                                    int32_t kernel, int32_t overlap, float *scratch,
                                    int32_t fill, void *workspace, size_t workspace_bytes,
                                    int64_t pair_capacity, int64_t checkpoint_capacity,
                                    const cbc_tuning *tuning, void *stream);

CBC_API int cbc_draw_lines_host_f64(double *host_out, int64_t n_frames, int64_t height,
                                    int64_t width, const double *lines, int64_t n_lines,
                                    const void *idxs, int32_t idx_bytes, double max_val,
                                    int32_t kernel, int32_t overlap, double *scratch,
                                    int32_t fill, void *workspace, size_t workspace_bytes,
                                    int64_t pair_capacity, int64_t checkpoint_capacity,
                                    const cbc_tuning *tuning, void *stream);

/* One Adam step on the (N, 5) float32 line parameters of a streak fit, in one kernel:
 * exp_avg = exp_avg + (1 - beta1)(grad - exp_avg),
 * exp_avg_sq = beta2 exp_avg_sq + (1 - beta2) grad^2,
 * params -= lr / (1 - beta1^step) * exp_avg / (sqrt(exp_avg_sq) / sqrt(1 - beta2^step) + eps),
 * then widths (column 4) are raised to min_width.  step counts from 1; the state
 * starts at zero.  No counterpart in the reference (new). */
CBC_API int cbc_adam_step_f32(float *params, const float *grad, float *exp_avg,
                              float *exp_avg_sq, int64_t n_lines, int64_t step, float lr,
                              float beta1, float beta2, float eps, float min_width,
                              void *stream);

/* accumulate_lines for 2-D lines.  Replaces bresenham.accumulate_lines
 * (_src/src/bresenham.cpp:301-327, accumulate_lines_nd_impl :151-259) and
 * cuda_draw_lines.accumulate_lines (_src/src/cuda_draw_lines.cu:1049-1057, 1077-1095).
 *
 * Line i belongs to term terms[i] (int32 or int64, term_bytes), term t to frame
 * frames[t] (frame_bytes); n_terms = length of frames.  Each term's lines are combined
 * with in_overlap (CBC_SUM / CBC_MAX) in a zeroed buffer, and every pixel the term
 * drew is merged into out[frames[t]] with out_overlap.  Errors seen on the device set
 * status flags and leave out untouched: frames outside [0, n_frames) set
 * CBC_ERR_INDEX (idx_min / idx_max hold the frames' range), a term outside
 * [0, n_terms) sets CBC_ERR_TERM (bad_line: the first such line).
 *
 * The mixed pairs (sum in / max out, max in / sum out) build each term's buffer in
 * shared memory, in up to eight partitions of its pixels.  Terms whose pixel estimate
 * needs more partitions keep their (term, pixel) values in a hash table of
 * `table_capacity` entries (0 or a power of two; 12 or 16 bytes each) in the
 * workspace; the call requires twice their estimated pairs and otherwise sets
 * CBC_ERR_CAPACITY with pairs_needed = the capacity to retry with, drawing nothing.
 * Calls without such terms need no table (table_capacity 0).  A checkpoint overflow
 * sets CBC_ERR_CAPACITY with checkpoints_needed.  The equal pairs use no table. */
CBC_API size_t cbc_accumulate_lines_workspace_size(int64_t n_lines, int64_t n_terms,
                                                   int64_t checkpoint_capacity,
                                                   int64_t table_capacity, int32_t elem_bytes);

CBC_API int cbc_accumulate_lines_f32(float *out, int64_t n_frames, int64_t height,
                                     int64_t width, const float *lines, int64_t n_lines,
                                     const void *terms, int32_t term_bytes, const void *frames,
                                     int32_t frame_bytes, int64_t n_terms, float max_val,
                                     int32_t kernel, int32_t in_overlap, int32_t out_overlap,
                                     void *workspace, size_t workspace_bytes,
                                     int64_t checkpoint_capacity, int64_t table_capacity,
                                     void *stream);

CBC_API int cbc_accumulate_lines_f64(double *out, int64_t n_frames, int64_t height,
                                     int64_t width, const double *lines, int64_t n_lines,
                                     const void *terms, int32_t term_bytes, const void *frames,
                                     int32_t frame_bytes, int64_t n_terms, double max_val,
                                     int32_t kernel, int32_t in_overlap, int32_t out_overlap,
                                     void *workspace, size_t workspace_bytes,
                                     int64_t checkpoint_capacity, int64_t table_capacity,
                                     void *stream);

/* draw_lines for 3-D lines into volumes.  Replaces the N = 3 instantiations of
 * bresenham.draw_lines (_src/src/bresenham.cpp:38-101 with draw_line_3d,
 * bresenham.hpp:389-430; dispatch on the line size :126-139) and of
 * cuda_draw_lines.draw_lines (_src/src/cuda_draw_lines.cu:925-933).
 * out: (n_frames, depth, height, width); lines: (n_lines, 7) rows
 * [x0, y0, z0, x1, y1, z1, width] (xyz order, z the slowest axis of a volume); idxs,
 * max_val, kernel, overlap and the status as for cbc_draw_lines_f32 (only the
 * checkpoint capacity applies; pairs_needed stays 0).  A voxel the reference's walk
 * visits twice is combined twice, as in the reference. */
CBC_API size_t cbc_draw_lines_3d_workspace_size(int64_t n_lines, int64_t checkpoint_capacity,
                                                int32_t elem_bytes);

CBC_API int cbc_draw_lines_3d_f32(float *out, int64_t n_frames, int64_t depth, int64_t height,
                                  int64_t width, const float *lines, int64_t n_lines,
                                  const void *idxs, int32_t idx_bytes, float max_val,
                                  int32_t kernel, int32_t overlap, void *workspace,
                                  size_t workspace_bytes, int64_t checkpoint_capacity,
                                  void *stream);

CBC_API int cbc_draw_lines_3d_f64(double *out, int64_t n_frames, int64_t depth, int64_t height,
                                  int64_t width, const double *lines, int64_t n_lines,
                                  const void *idxs, int32_t idx_bytes, double max_val,
                                  int32_t kernel, int32_t overlap, void *workspace,
                                  size_t workspace_bytes, int64_t checkpoint_capacity,
                                  void *stream);

/* accumulate_lines for 3-D lines into volumes (N = 3 of bresenham.cpp:151-259;
 * cuda_draw_lines.cu:1034-1042), with the arguments, status and table_capacity rule
 * of cbc_accumulate_lines_f32 plus the volume depth (eight partitions of a 8192-voxel
 * shared-memory table per term before a term goes to the workspace table).  The
 * checkpoint capacity counts one checkpoint per long-axis column of each line. */
CBC_API size_t cbc_accumulate_lines_3d_workspace_size(int64_t n_lines, int64_t n_terms,
                                                      int64_t checkpoint_capacity,
                                                      int64_t table_capacity,
                                                      int32_t elem_bytes);

CBC_API int cbc_accumulate_lines_3d_f32(float *out, int64_t n_frames, int64_t depth,
                                        int64_t height, int64_t width, const float *lines,
                                        int64_t n_lines, const void *terms, int32_t term_bytes,
                                        const void *frames, int32_t frame_bytes,
                                        int64_t n_terms, float max_val, int32_t kernel,
                                        int32_t in_overlap, int32_t out_overlap,
                                        void *workspace, size_t workspace_bytes,
                                        int64_t checkpoint_capacity, int64_t table_capacity,
                                        void *stream);

CBC_API int cbc_accumulate_lines_3d_f64(double *out, int64_t n_frames, int64_t depth,
                                        int64_t height, int64_t width, const double *lines,
                                        int64_t n_lines, const void *terms, int32_t term_bytes,
                                        const void *frames, int32_t frame_bytes,
                                        int64_t n_terms, double max_val, int32_t kernel,
                                        int32_t in_overlap, int32_t out_overlap,
                                        void *workspace, size_t workspace_bytes,
                                        int64_t checkpoint_capacity, int64_t table_capacity,
                                        void *stream);

/* Adjoint of cbc_draw_lines_3d_* (no counterpart in the reference): grad_lines
 * (n_lines, 7) = the gradient of sum(grad_out * volumes) with respect to
 * (x0, y0, z0, x1, y1, z1, width), over exactly the voxel visits of the forward (a
 * voxel the walk visits twice counts twice under sum overlap, as its value does).
 * Max overlap gives each voxel's gradient to its winner only, the smallest line whose
 * value equals `image` (the forward's result) and exceeds `out0` (the volumes before
 * drawing; NULL: zeros); `winner` (n_frames, depth, height, width) int32 comes back
 * holding those winners (0x7f7f7f7f where no line drew the value).  Workspace from
 * cbc_draw_lines_3d_backward_workspace_size; capacity and errors as the forward. */
CBC_API size_t cbc_draw_lines_3d_backward_workspace_size(int64_t n_lines,
                                                         int64_t checkpoint_capacity,
                                                         int32_t elem_bytes);

CBC_API int cbc_draw_lines_3d_backward_f32(const float *grad_out, int64_t n_frames,
                                           int64_t depth, int64_t height, int64_t width,
                                           const float *lines, int64_t n_lines,
                                           const void *idxs, int32_t idx_bytes, float max_val,
                                           int32_t kernel, int32_t overlap, const float *image,
                                           const float *out0, int32_t *winner,
                                           float *grad_lines, void *workspace,
                                           size_t workspace_bytes, int64_t checkpoint_capacity,
                                           void *stream);

CBC_API int cbc_draw_lines_3d_backward_f64(const double *grad_out, int64_t n_frames,
                                           int64_t depth, int64_t height, int64_t width,
                                           const double *lines, int64_t n_lines,
                                           const void *idxs, int32_t idx_bytes,
                                           double max_val, int32_t kernel, int32_t overlap,
                                           const double *image, const double *out0,
                                           int32_t *winner, double *grad_lines,
                                           void *workspace, size_t workspace_bytes,
                                           int64_t checkpoint_capacity, void *stream);

/* Wait for `stream` and copy the device status of the last call that used
 * `workspace` into *status.  Returns CBC_OK or CBC_ERR_CUDA. */
CBC_API int cbc_read_status(const void *workspace, cbc_status *status, void *stream);

/* The same status without waiting: cbc_copy_status_async enqueues on `stream` a copy
 * of the device status block (cbc_status_bytes() bytes) into host memory `dst`
 * (page-locked for an asynchronous copy); once the stream has passed it,
 * cbc_decode_status turns those bytes into *status.  For callers that run several
 * calls on several streams and check them all at one synchronisation point.
 * No counterpart in the reference (new). */
CBC_API size_t cbc_status_bytes(void);
CBC_API int cbc_copy_status_async(const void *workspace, void *dst, void *stream);
CBC_API int cbc_decode_status(const void *src, cbc_status *status);

/* Per-stage device time of the calls made while profiling is on, from CUDA events
 * recorded on each call's stream around its kernels (no effect on results). */
typedef struct cbc_profile {
    int32_t calls;         /* calls measured since the last reset                    */
    int32_t launches;      /* kernels the library launched since the last reset, in
                              all calls (forward and backward, profiled or not)     */
    double ms_prep;        /* status init + line records + tile counts (tiles), or
                              status init + line records + walk checkpoints (lines) */
    double ms_offsets;     /* bin offsets (tiles; 0 for lines)                       */
    double ms_fill;        /* (line, tile) pair fill (tiles; 0 for lines)            */
    double ms_render;      /* render_kernel (tiles) or segments_kernel (lines)       */
} cbc_profile;

/* Turn the per-stage event timing on (1) or off (0); returns the previous state. */
CBC_API int cbc_profile_enable(int32_t on);

/* Wait for the recorded events, add their times into *profile (zeroed first when
 * `reset` is 1, which also clears the accumulated calls).  Returns CBC_OK or
 * CBC_ERR_CUDA. */
CBC_API int cbc_profile_read(cbc_profile *profile, int32_t reset);

/* Message of the last host-side error on the calling thread ("" if none). */
CBC_API const char *cbc_last_error(void);

/* Library version string. */
CBC_API const char *cbc_version(void);

#ifdef __cplusplus
}
#endif

#endif /* CBC_DRAW_LINES_H */
