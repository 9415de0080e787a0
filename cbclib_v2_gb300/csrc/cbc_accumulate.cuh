/*
 * cbc_accumulate.cuh — pieces of accumulate_lines shared by the 2-D and 3-D paths
 * (cbc_accumulate.cu, cbc_lines3d.cu): the overlap pairs, the (term, pixel) hash table,
 * term and frame validation, and the merge of the table into the frames.
 */
#ifndef CBC_ACCUMULATE_CUH
#define CBC_ACCUMULATE_CUH

#include "cbc_common.cuh"

namespace cbc {

/* bit 0: terms combine their lines by max; bit 1: terms merge into out by max
 * (the Update encoding of bresenham.cpp:304-307) */
enum : int { kAccSumSum = 0, kAccMaxSum = 1, kAccSumMax = 2, kAccMaxMax = 3 };

constexpr unsigned long long kEmptyKey = ~0ull;
constexpr int kMaxProbe = 64;

/* splitmix64's finaliser (Steele, Lea and Flood 2014) as the table's hash */
__device__ __forceinline__ unsigned long long mix64(unsigned long long x)
{
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

/* std::max(buffer, v) with buffer starting at +0, as an atomic on the slot's value */
template <typename T>
__device__ __forceinline__ void term_combine_max(T *slot, T v);

template <>
__device__ __forceinline__ void term_combine_max<float>(float *slot, float v)
{
    /* the slot holds +0 or a positive value: only v > 0 can change it, and positive
     * floats order as their bit patterns (NaN and negative v leave it unchanged) */
    if (v > 0.0f) atomicMax(reinterpret_cast<int *>(slot), __float_as_int(v));
}

template <>
__device__ __forceinline__ void term_combine_max<double>(double *slot, double v)
{
    if (v > 0.0) atomicMax(reinterpret_cast<long long *>(slot), __double_as_longlong(v));
}

/* combine v into the table entry of (term, pixel): claim an empty slot or find the
 * key along at most kMaxProbe slots of linear probing; a full path sets
 * CBC_ERR_CAPACITY and asks for four times the capacity */
template <typename T, int IN_MAX>
__device__ __forceinline__ void table_combine(unsigned long long *keys, T *vals,
                                              unsigned long long mask, int term,
                                              long long pix, T v, DevStatus *st)
{
    const unsigned long long key = ((unsigned long long)(unsigned)term << 32) |
                                   (unsigned long long)(unsigned)pix;
    unsigned long long h = mix64(key) & mask;
    for (int probe = 0; probe < kMaxProbe; probe++) {
        unsigned long long k = *reinterpret_cast<volatile unsigned long long *>(keys + h);
        if (k == kEmptyKey) k = atomicCAS(keys + h, kEmptyKey, key);
        if (k == kEmptyKey || k == key) {
            if (IN_MAX) term_combine_max(vals + h, v);
            else atomicAdd(vals + h, v);
            return;
        }
        h = (h + 1) & mask;
    }
    atomicOr(&st->flags, 1 << CBC_ERR_CAPACITY);
    atomicMax(&st->pairs, 4ull * (mask + 1));
}

/* each term's first slot in the line list: block scan, one cursor atomic per block */
static __global__ void __launch_bounds__(kThreads)
term_offsets_kernel(const int *__restrict__ tcount, int *__restrict__ toff,
                    int *__restrict__ tfill, long long n_terms, unsigned long long *cursor)
{
    __shared__ int warp_sums[kThreads / 32];
    __shared__ unsigned long long block_base;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int c = t < n_terms ? tcount[t] : 0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = c;
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int v = lane < kThreads / 32 ? warp_sums[lane] : 0;
        int sum = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, sum, o);
            if (lane >= o) sum += u;
        }
        if (lane < kThreads / 32) warp_sums[lane] = sum - v;
        if (lane == kThreads / 32 - 1) block_base = atomicAdd(cursor, (unsigned long long)sum);
    }
    __syncthreads();
    if (t >= n_terms) return;
    const int o = (int)(block_base + (unsigned long long)(warp_sums[wid] + incl - c));
    toff[t] = o;
    tfill[t] = o;
}

/* terms whose pixel estimate exceeds `limit` (more partitions of a shared-memory
 * table than the term renders take) go through the workspace table; their count and
 * estimated pairs size it */
static __global__ void __launch_bounds__(kThreads)
term_class_kernel(const int *__restrict__ tcount, const float *__restrict__ test,
                   long long n_terms, float limit, int *__restrict__ tbig, int *nbig,
                   float *big_est)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_terms) return;
    const bool big = tcount[t] > 0 && test[t] > limit;
    tbig[t] = big ? 1 : 0;
    if (big) {
        atomicAdd(nbig, 1);
        atomicAdd(big_est, test[t]);
    }
}

/* whether the table pass has work: false when no term goes through the workspace
 * table, or when the table holds fewer than twice their estimated pairs (rounded up to
 * a power of two, at least 1024); the latter sets CBC_ERR_CAPACITY with that capacity
 * as pairs_needed, so the call draws nothing and can be retried */
__device__ __forceinline__ bool table_terms_fit(const int *nbig, const float *big_est,
                                                long long capacity, DevStatus *st)
{
    if (*nbig == 0) return false;
    unsigned long long need = 1024;
    while ((float)need < 2.0f * *big_est && need < (1ull << 40)) need <<= 1;
    if ((unsigned long long)capacity >= need) return true;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicOr(&st->flags, 1 << CBC_ERR_CAPACITY);
        atomicMax(&st->pairs, need);
    }
    return false;
}

/* the partition of a pixel or voxel index: hash bits independent of the table slot's
 * (the shared-memory term renders take a term's pixels in partitions) */
__device__ __forceinline__ unsigned part_hash(unsigned k)
{
    unsigned x = k * 0x85ebca6bu;
    return x ^ (x >> 16);
}

/* every frames[t] in [0, n_frames) (bresenham.cpp:23-36: "frames range (min, max) is
 * outside of (0, n_frames)"); the int32 copy feeds the merge */
template <typename FI>
__global__ void __launch_bounds__(kThreads)
frames_check_kernel(const FI *__restrict__ frames, long long n_terms, long long n_frames,
                    int *__restrict__ frame_of_term, DevStatus *st)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = t < n_terms;
    const long long f = in ? (long long)frames[t] : 0;
    warp_minmax(f, in, st);
    if (!in) return;
    if (f < 0 || f >= n_frames) atomicOr(&st->flags, 1 << CBC_ERR_INDEX);
    frame_of_term[t] = (f >= 0 && f < n_frames) ? (int)f : 0;
}

/* per line: its term (bresenham.cpp:182-188: "Term index t is out of range (0, T)")
 * and its frame */
template <typename TI>
__global__ void __launch_bounds__(kThreads)
term_frames_kernel(const TI *__restrict__ terms, const int *__restrict__ frame_of_term,
                   long long n_lines, long long n_terms, int *__restrict__ term_of_line,
                   int *__restrict__ frame_of_line, DevStatus *st)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_lines) return;
    const long long t = (long long)terms[i];
    if (t < 0 || t >= n_terms) {
        atomicOr(&st->flags, 1 << CBC_ERR_TERM);
        atomicMin(&st->bad_line, (unsigned long long)i);
        term_of_line[i] = 0;
        frame_of_line[i] = 0;
        return;
    }
    term_of_line[i] = (int)t;
    frame_of_line[i] = frame_of_term[t];
}

/* the table's entries merged into out with out_overlap (sum: out = v + out;
 * max: out = std::max(out, v)); nothing when the call has failed */
template <typename T, int OUT_MAX>
__global__ void __launch_bounds__(kThreads)
merge_kernel(T *__restrict__ out, const unsigned long long *__restrict__ keys,
             const T *__restrict__ vals, long long cap, const int *__restrict__ frame_of_term,
             long long frame_px, const DevStatus *st)
{
    if (st->flags & kFatal) return;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < cap;
         i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long k = keys[i];
        if (k == kEmptyKey) continue;
        const int term = (int)(k >> 32);
        T *dst = out + (long long)frame_of_term[term] * frame_px + (long long)(k & 0xffffffffull);
        if (OUT_MAX) global_combine_max(dst, vals[i]);
        else atomicAdd(dst, vals[i]);
    }
}

struct AccLayout {
    size_t status, recs, cks, frame_of_line, term_of_line, frame_of_term, keys, vals;
    size_t tcount, toff, tfill, test, tlines, tbig, counters, total;
};

/* the counters block after `counters`: the line-list cursor (unsigned long long), the
 * number of table terms (int) and their estimated pairs (float) */
inline AccLayout acc_layout(long long n_lines, long long n_terms, long long ck_capacity,
                     long long table_capacity, size_t rec_bytes, size_t ck_bytes, size_t elem)
{
    auto up = [](size_t v) { return (v + 255) / 256 * 256; };
    AccLayout L;
    size_t off = 0;
    L.status = off;        off = up(off + sizeof(DevStatus));
    L.recs = off;          off = up(off + rec_bytes * (size_t)n_lines);
    L.cks = off;           off = up(off + ck_bytes * (size_t)ck_capacity);
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
    L.counters = off;      off = up(off + 16);
    L.total = off;
    return L;
}

/* frames_check_kernel over the n_terms entries of `frames` (int32 or int64) */
inline cudaError_t launch_frames_check(const void *frames, int frame_bytes, long long n_terms,
                                       long long n_frames, int *frame_of_term, DevStatus *st,
                                       cudaStream_t s)
{
    if (n_terms <= 0) return cudaSuccess;
    const unsigned nb = (unsigned)((n_terms + kThreads - 1) / kThreads);
    if (frame_bytes == 8)
        frames_check_kernel<int64_t><<<nb, kThreads, 0, s>>>(
            static_cast<const int64_t *>(frames), n_terms, n_frames, frame_of_term, st);
    else
        frames_check_kernel<int32_t><<<nb, kThreads, 0, s>>>(
            static_cast<const int32_t *>(frames), n_terms, n_frames, frame_of_term, st);
    note_launches(1);
    return cudaGetLastError();
}

/* term_frames_kernel over the n_lines entries of `terms` (int32 or int64) */
inline cudaError_t launch_term_frames(const void *terms, int term_bytes, const int *frame_of_term,
                                      long long n_lines, long long n_terms, int *term_of_line,
                                      int *frame_of_line, DevStatus *st, cudaStream_t s)
{
    const unsigned nb = (unsigned)((n_lines + kThreads - 1) / kThreads);
    if (term_bytes == 8)
        term_frames_kernel<int64_t><<<nb, kThreads, 0, s>>>(
            static_cast<const int64_t *>(terms), frame_of_term, n_lines, n_terms, term_of_line,
            frame_of_line, st);
    else
        term_frames_kernel<int32_t><<<nb, kThreads, 0, s>>>(
            static_cast<const int32_t *>(terms), frame_of_term, n_lines, n_terms, term_of_line,
            frame_of_line, st);
    note_launches(1);
    return cudaGetLastError();
}

/* an empty table: every key kEmptyKey, every value +0 */
template <typename T>
cudaError_t clear_table(unsigned long long *keys, T *vals, long long cap, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(keys, 0xff, sizeof(unsigned long long) * (size_t)cap, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(vals, 0, sizeof(T) * (size_t)cap, s);
    return e;
}

/* merge_kernel on a grid of at most 8 CTAs per SM striding over the table */
template <typename T>
cudaError_t launch_merge(T *out, const unsigned long long *keys, const T *vals, long long cap,
                         const int *frame_of_term, long long frame_px, bool out_max,
                         const DevStatus *st, cudaStream_t s)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long blocks = (cap + kThreads - 1) / kThreads;
    const long long most = (long long)(sms > 0 ? sms : 132) * 8;
    if (blocks > most) blocks = most;
    if (blocks < 1) blocks = 1;
    if (out_max)
        merge_kernel<T, 1><<<(unsigned)blocks, kThreads, 0, s>>>(out, keys, vals, cap,
                                                                 frame_of_term, frame_px, st);
    else
        merge_kernel<T, 0><<<(unsigned)blocks, kThreads, 0, s>>>(out, keys, vals, cap,
                                                                 frame_of_term, frame_px, st);
    note_launches(1);
    return cudaGetLastError();
}

}  // namespace cbc

#endif /* CBC_ACCUMULATE_CUH */
