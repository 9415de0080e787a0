/* Host build of the GPU kernels' float emulation (cbclib_v2_gb300/csrc/exact.cuh) so the
 * tests can compare it with the oracle on the CPU.  Built with -ffp-contract=off. */
#include <stdint.h>
static long long cbc_slow_count = 0;
#define CBC_SLOW_HOOK() (cbc_slow_count++)
#include "exact.cuh"

/* evaluations that left the float pair path since the last call */
long long exact_take_slow_count(void)
{
    long long c = cbc_slow_count;
    cbc_slow_count = 0;
    return c;
}

void exact_profile_batch(int kernel, const float *x, float *out, int64_t n)
{
    for (int64_t i = 0; i < n; i++) out[i] = cbc_profile_f32(kernel, x[i]);
}

void exact_pixel_error_batch(const float *te, const float *ne, const float *len,
                             const float *width, float *out, int64_t n)
{
    for (int64_t i = 0; i < n; i++) {
        float w = width[i];
        if (!(w > 0.0f)) { out[i] = 1.0f / 0.0f; continue; }
        float nf = cbc_normal_term(ne[i], len[i]);
        out[i] = cbc_pixel_error(te[i], nf, len[i], len[i] * len[i], w * w);
    }
}

/* fraction of evaluations that leave the float fast path */
void exact_fast_path_stats(int which, const float *x, int64_t n, int64_t *slow)
{
    int64_t s = 0;
    for (int64_t i = 0; i < n; i++) {
        float r;
        if (which == 0) {   /* one_minus_sq */
            float v = x[i];
            float p = v * v, pe = fmaf(v, v, -p), t = 1.0f - p, z = t - 1.0f, e = -p - z;
            s += !cbc_ff_round(t, e - pe, &r);
        }
    }
    *slow = s;
}

/* the reciprocal-based division path used when len and ww are in [2^-60, 2^60] */
void exact_pixel_error_r_batch(const float *te, const float *ne, const float *len,
                               const float *width, float *out, int64_t n)
{
    for (int64_t i = 0; i < n; i++) {
        float w = width[i], l = len[i];
        float ww = w * w, rl = 1.0f / l, rww = 1.0f / ww;
        if (!(w > 0.0f) || !(l >= CBC_DIV_LO && l <= CBC_DIV_HI && ww >= CBC_DIV_LO && ww <= CBC_DIV_HI)) {
            out[i] = -1.0f;   /* not a fast-path input */
            continue;
        }
        float nf = cbc_normal_term_r(ne[i], l, rl);
        out[i] = cbc_pixel_error_r(te[i], nf, l, l * l, ww, rl, rww);
    }
}

void exact_div_batch(const float *a, const float *b, float *out, int64_t n)
{
    for (int64_t i = 0; i < n; i++) out[i] = cbc_div(a[i], b[i], 1.0f / b[i]);
}

/* BresenhamPlotter::normal_error of 3-D positions; use_r selects the reciprocal path
 * (-1 where len is outside its range) */
void exact_normal_error3_batch(const float *n0, const float *n1, const float *n2,
                               const float *len, float *out, int64_t n, int use_r)
{
    for (int64_t i = 0; i < n; i++) {
        float l = len[i];
        if (use_r) {
            if (!(l >= CBC_DIV_LO && l <= CBC_DIV_HI)) { out[i] = -1.0f; continue; }
            out[i] = cbc_normal_error3_r(n0[i], n1[i], n2[i], l, 1.0f / l);
        } else {
            out[i] = cbc_normal_error3(n0[i], n1[i], n2[i], l);
        }
    }
}

void exact_ddiv_batch(const double *a, const double *b, double *out, int64_t n)
{
    for (int64_t i = 0; i < n; i++) out[i] = cbc_ddiv(a[i], b[i], 1.0 / b[i]);
}
