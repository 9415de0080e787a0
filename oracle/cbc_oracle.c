/*
 * ORACLE — test infrastructure, not product code.
 *
 * CPU restatement of the reference project's `draw_lines` / `accumulate_lines` CPU path
 * (cbclib_v2/_src/src/bresenham.{hpp,cpp}), used only as the checker of the GPU
 * kernels by tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py.
 * It is pinned bit-for-bit against the reference module itself (oracle/build_ref.sh)
 * and against golden fixtures generated from it (tests/golden/make_golden.py).
 *
 * Exported entry points (plain C ABI for ctypes):
 *   cbc_oracle_draw_lines_{f32,f64}        draw_lines_nd_impl, bresenham.cpp:38-101
 *   cbc_oracle_accumulate_lines_{f32,f64}  accumulate_lines_nd_impl, bresenham.cpp:151-259
 *   cbc_oracle_profile_{f32,f64}           kernel_traits, include.hpp:447-468
 *   cbc_oracle_pixel_error_f32             BresenhamPlotter::error, bresenham.hpp:291-296
 * Return codes: 0 ok, 1 invalid argument, 2 index out of range.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OT float
#define OSFX f32
#include "oracle_impl.h"
#undef OT
#undef OSFX

#define OT double
#define OSFX f64
#include "oracle_impl.h"
#undef OT
#undef OSFX

float cbc_oracle_profile_f32(int kernel, float x) { return oprofile_f32(kernel, x); }
double cbc_oracle_profile_f64(int kernel, double x) { return oprofile_f64(kernel, x); }

/* the per-pixel error of a 2-D walk position, from its tangent/normal errors */
float cbc_oracle_pixel_error_f32(float te, float ne, float len, float width)
{
    oplot_f32 p;
    oiter_f32 it;
    memset(&p, 0, sizeof p);
    memset(&it, 0, sizeof it);
    p.n = 2;
    p.len = len;
    it.te = te;
    it.ne[0] = ne;
    return oerror_f32(&p, &it, width);
}

/* batch forms for the tests of the float emulation in the GPU kernels */
void cbc_oracle_profile_batch_f32(int kernel, const float *x, float *out, int64_t n)
{
    for (int64_t i = 0; i < n; i++) out[i] = oprofile_f32(kernel, x[i]);
}

void cbc_oracle_pixel_error_batch_f32(const float *te, const float *ne, const float *len,
                                      const float *width, float *out, int64_t n)
{
    for (int64_t i = 0; i < n; i++) out[i] = cbc_oracle_pixel_error_f32(te[i], ne[i], len[i], width[i]);
}
