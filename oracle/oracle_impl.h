/*
 * ORACLE — test infrastructure only.  Included twice by cbc_oracle.c with
 *   OT   = the scalar type of the reference overload (float or double),
 *   OSFX = the symbol suffix (f32 / f64).
 *
 * A plain-C restatement of the reference CPU rasteriser
 *   cbclib_v2/_src/src/bresenham.hpp   (BaseError :39-65, TangentError :67-81,
 *                                       NormalError :83-112, LineIterator :117-231,
 *                                       BresenhamPlotter :233-348, draw_line_2d :352-383,
 *                                       draw_line_3d :389-430)
 *   cbclib_v2/_src/src/bresenham.cpp   (fill_indices :5-20, check_indices :22-36,
 *                                       draw_lines_nd_impl :38-101, accumulate_lines_nd_impl
 *                                       :151-259)
 *   cbclib_v2/_src/src/include.hpp     (kernel_traits :447-468)
 *   cbclib_v2/_src/src/geometry.hpp    (dot :250-256, magnitude/amplitude :260-272,
 *                                       PointND::round :212-217, UniquePairs :403-448)
 *
 * Arithmetic follows the reference operation by operation, including its C++ type
 * promotions: std::pow(T, int) is evaluated in double (C++11 [c.math]), so squared terms,
 * the per-pixel error sum and three of the five profiles round through double before
 * they are converted back to OT.  Compiled with -ffp-contract=off so no FMA contraction
 * changes a rounding (the reference is built without -march on x86-64, which has no FMA).
 */

#define OCAT2(a, b) a##_##b
#define OCAT(a, b) OCAT2(a, b)
#define OF(name) OCAT(name, OSFX)

/* one iterator of the N-dimensional Bresenham walk (bresenham.hpp:117-231) */
typedef struct {
    long step[3];
    long cur[3];
    int next[3];
    OT te;          /* TangentError::error */
    OT ne[3];       /* NormalError::error, one per axis pair */
} OF(oiter);

typedef struct {
    int n;                 /* 2 or 3 */
    int axis;              /* long axis */
    OT pt0[3], pt1[3];
    OT tau[3];             /* tangent pt1 - pt0 (TangentError::derror) */
    OT nrm[3][3];          /* normal of each pair (NormalError::derror) */
    OT len;                /* TangentError::length = amplitude(tau) */
    long mpt0[3], mpt1[3]; /* walk start, walk end (+step) */
    long step[3];
} OF(oplot);

/* UniquePairs<N> (geometry.hpp:403-448): N=2 -> (0,1); N=3 -> (0,1),(0,2),(1,2) */
static const int OF(pair_a)[3] = {0, 0, 1};
static const int OF(pair_b)[3] = {1, 2, 2};

static inline int OF(npairs)(int n) { return n * (n - 1) / 2; }

static inline OT OF(omax)(OT a, OT b) { return (a < b) ? b : a; }   /* std::max */

/* dot(a, b) with T accumulation in index order: res = 0; res += a[i] * b[i] */
static inline OT OF(odot)(const OT *a, const OT *b, int n)
{
    OT r = (OT)0;
    for (int i = 0; i < n; i++) r = r + a[i] * b[i];
    return r;
}

/* LineIterator::update (bresenham.hpp:205-220) with NormalError::is_next (:98-111) */
static void OF(oupdate)(const OF(oplot) *p, OF(oiter) *it)
{
    for (int i = 0; i < p->n; i++) it->next[i] = it->step[i] != 0;
    for (int k = 0; k < OF(npairs)(p->n); k++) {
        int a1 = OF(pair_a)[k], a2 = OF(pair_b)[k];
        if (it->step[a1] && it->step[a2]) {
            OT e = it->ne[k];
            OT ex = e + (OT)it->step[a1] * p->nrm[k][a1];
            OT ey = e + (OT)it->step[a2] * p->nrm[k][a2];
            OT exy = ex + (OT)it->step[a2] * p->nrm[k][a2];
            int f, s;
            if (fabs(ey) < fabs(ex)) {
                if (fabs(exy) < fabs(ey)) { f = 1; s = 1; } else { f = 0; s = 1; }
            } else {
                if (fabs(exy) < fabs(ex)) { f = 1; s = 1; } else { f = 1; s = 0; }
            }
            it->next[a1] &= f;
            it->next[a2] &= s;
        }
    }
}

/* LineIterator::increment (bresenham.hpp:195-203) */
static inline void OF(oincrement)(const OF(oplot) *p, OF(oiter) *it, long x, int axis)
{
    it->cur[axis] += x;
    it->te = it->te + (OT)x * p->tau[axis];
    for (int k = 0; k < OF(npairs)(p->n); k++) {
        if (OF(pair_a)[k] == axis || OF(pair_b)[k] == axis)
            it->ne[k] = it->ne[k] + (OT)x * p->nrm[k][axis];
    }
}

static inline void OF(oadvance)(const OF(oplot) *p, OF(oiter) *it)        /* operator++ */
{
    for (int i = 0; i < p->n; i++) if (it->next[i]) OF(oincrement)(p, it, it->step[i], i);
    OF(oupdate)(p, it);
}

static inline void OF(omove)(const OF(oplot) *p, OF(oiter) *it, int axis)  /* move */
{
    OF(oincrement)(p, it, it->step[axis], axis);
    OF(oupdate)(p, it);
}

static inline OF(oiter) OF(ocollapse)(const OF(oplot) *p, const OF(oiter) *src, int axis)
{
    OF(oiter) it = *src;
    it.step[axis] = 0;
    OF(oupdate)(p, &it);
    return it;
}

/* any coordinate equal to the end point terminates the walk (LineIterator::operator==) */
static inline int OF(oat_end)(const OF(oplot) *p, const OF(oiter) *it)
{
    for (int i = 0; i < p->n; i++) if (it->cur[i] == p->mpt1[i]) return 1;
    return 0;
}

/* BresenhamPlotter::normal_error (bresenham.hpp:284-289): T accumulator fed with doubles */
static inline OT OF(onormal_error)(const OF(oplot) *p, const OF(oiter) *it)
{
    OT err = (OT)0;
    for (int k = 0; k < OF(npairs)(p->n); k++) {
        double b = (double)(it->ne[k] / p->len);
        err = (OT)((double)err + b * b);
    }
    return err;
}

/* BresenhamPlotter::error (bresenham.hpp:291-296) */
static inline OT OF(oerror)(const OF(oplot) *p, const OF(oiter) *it, OT width)
{
    if (width <= (OT)0) return (OT)INFINITY;
    OT te = it->te;
    OT ta = OF(omax)(OF(omax)(-te, te - p->len * p->len), (OT)0);
    double a = (double)(ta / p->len);
    double e = a * a + (double)OF(onormal_error)(p, it);
    return (OT)(e / (double)(width * width));
}

/* kernel_traits<T> (include.hpp:447-468); x = sqrt(error) in [0, 1] */
static inline OT OF(oprofile)(int kernel, OT x)
{
    switch (kernel) {
    case 0: {   /* biweight: T(0.9375) * pow(max<T>(1 - pow(x, 2), T()), 2) */
        double xd = (double)x;
        OT m = OF(omax)((OT)(1.0 - xd * xd), (OT)0);
        double md = (double)m;
        return (OT)((double)(OT)0.9375 * (md * md));
    }
    case 1: {   /* gaussian: M_1_SQRT2PI * exp(-pow(3 * x, 2) / 2) for |x| <= 1 */
        if (fabs(x) <= (OT)1.0) {
            double y = (double)((OT)3 * x);
            return (OT)(0.3989422804014327 * exp(-(y * y) / 2));
        }
        return (OT)0;
    }
    case 2: {   /* parabolic: T(0.75) * max<T>(1 - pow(x, 2), T()) */
        double xd = (double)x;
        OT m = OF(omax)((OT)(1.0 - xd * xd), (OT)0);
        return (OT)0.75 * m;
    }
    case 3:     /* rectangular */
        return (fabs(x) <= (OT)1.0) ? (OT)1.0 : (OT)0;
    default:    /* triangular: max<T>(1 - |x|, 0) */
        return OF(omax)((OT)1.0 - (OT)fabs(x), (OT)0);
    }
}

/* BresenhamPlotter(line, offset) constructor (bresenham.hpp:243-253) and the error
 * origins of begin() (:255-263).  Returns 0 when the walk would not be defined (the
 * reference reaches undefined behaviour there and in practice draws nothing). */
static int OF(oplot_init)(OF(oplot) *p, const OT *ln, int n, OF(oiter) *begin)
{
    p->n = n;
    for (int i = 0; i < n; i++) { p->pt0[i] = ln[i]; p->pt1[i] = ln[n + i]; }
    OT width = ln[2 * n];
    for (int i = 0; i < 2 * n + 1; i++) if (!isfinite(ln[i])) return 0;
    for (int i = 0; i < n; i++) p->tau[i] = p->pt1[i] - p->pt0[i];
    /* long_axis: first index of max |tau| */
    int ax = 0;
    for (int i = 1; i < n; i++) if (fabs(p->tau[ax]) < fabs(p->tau[i])) ax = i;
    p->axis = ax;
    OT mag = OF(odot)(p->tau, p->tau, n);
    OT amp = (OT)sqrt(mag);
    p->len = amp;
    if (!(amp > (OT)0)) return 0;   /* zero-length: error is NaN at every pixel */
    OT ceilw = (OT)ceil(width) + (OT)1;
    if (!(fabs(ceilw) < (OT)1e9)) return 0;
    long offset = (long)ceilw;
    OT tn[3];
    for (int i = 0; i < n; i++) tn[i] = p->tau[i] / amp;
    OT scale = (OT)fabs((OT)offset / tn[ax]);
    for (int i = 0; i < n; i++) {
        p->step[i] = (p->pt1[i] >= p->pt0[i]) ? 1 : -1;
        OT a = (OT)round(p->pt0[i] - scale * tn[i]);
        OT b = (OT)round(p->pt1[i] + scale * tn[i]);
        if (!(fabs(a) < (OT)4e18) || !(fabs(b) < (OT)4e18)) return 0;
        p->mpt0[i] = (long)a;
        p->mpt1[i] = (long)b + p->step[i];
    }
    for (int k = 0; k < 3; k++) for (int i = 0; i < 3; i++) p->nrm[k][i] = (OT)0;
    for (int k = 0; k < OF(npairs)(n); k++) {
        int a1 = OF(pair_a)[k], a2 = OF(pair_b)[k];
        p->nrm[k][a1] = p->pt1[a2] - p->pt0[a2];
        p->nrm[k][a2] = p->pt0[a1] - p->pt1[a1];
    }
    /* begin(): errors at m_pt0 relative to pt0 */
    OT d[3];
    for (int i = 0; i < n; i++) d[i] = (OT)p->mpt0[i] - p->pt0[i];
    for (int i = 0; i < n; i++) { begin->step[i] = p->step[i]; begin->cur[i] = p->mpt0[i]; }
    begin->te = OF(odot)(p->tau, d, n);
    for (int k = 0; k < OF(npairs)(n); k++) begin->ne[k] = OF(odot)(p->nrm[k], d, n);
    OF(oupdate)(p, begin);
    return 1;
}

/* a visited pixel: BresenhamPlotter::error then the draw_pixel lambda of
 * draw_lines_nd_impl (bresenham.cpp:78-87) */
typedef struct {
    int n;
    const int64_t *shape;   /* spatial shape, C order (H, W) or (D, H, W) */
    OT width;
    void (*emit)(void *ctx, int64_t flat, OT error);
    void *ctx;
} OF(osink);

static inline void OF(ovisit)(const OF(oplot) *p, const OF(oiter) *it, const OF(osink) *s)
{
    OT err = OF(oerror)(p, it, s->width);
    if (!(err <= (OT)1.0)) return;
    int64_t flat = 0;
    for (int i = p->n - 1; i >= 0; i--) {        /* point is xyz, shape is zyx */
        long c = it->cur[i];
        int64_t ext = s->shape[p->n - 1 - i];
        if (c < 0 || c >= ext) return;
        flat = flat * ext + c;
    }
    s->emit(s->ctx, flat, err);
}

/* draw_line_2d (bresenham.hpp:352-383) */
static void OF(odraw_2d)(const OF(oplot) *p, OF(oiter) it, const OF(osink) *s)
{
    OT ww = s->width * s->width;
    int ax = p->axis, sh = (ax + 1) % 2;
    for (; !OF(oat_end)(p, &it); OF(oadvance)(p, &it)) {
        if (!it.next[ax]) continue;
        OF(ovisit)(p, &it, s);
        OF(oiter) ix = OF(ocollapse)(p, &it, ax);
        for (OF(oadvance)(p, &ix); OF(onormal_error)(p, &ix) < ww; OF(oadvance)(p, &ix))
            OF(ovisit)(p, &ix, s);
        ix = OF(ocollapse)(p, &it, ax);
        ix.step[sh] *= -1;
        OF(oupdate)(p, &ix);
        for (OF(oadvance)(p, &ix); OF(onormal_error)(p, &ix) < ww; OF(oadvance)(p, &ix))
            OF(ovisit)(p, &ix, s);
    }
}

/* draw_line_3d (bresenham.hpp:389-430) */
static void OF(odraw_3d)(const OF(oplot) *p, OF(oiter) it, const OF(osink) *s)
{
    OT ww = s->width * s->width;
    int ax = p->axis;
    int ax1 = (ax + 1) % 3, ax2 = (ax + 2) % 3;
    for (; !OF(oat_end)(p, &it); OF(oadvance)(p, &it)) {
        if (!it.next[ax]) continue;
        OF(ovisit)(p, &it, s);
        for (int q = 0; q < 4; q++) {
            OF(oiter) ixy = OF(ocollapse)(p, &it, ax);
            if (q & 1) ixy.step[ax1] *= -1;
            if (q >> 1) ixy.step[ax2] *= -1;
            OF(oupdate)(p, &ixy);
            int mv = (1 + ((q & 1) ^ (q >> 1)) == 1) ? ax1 : ax2;
            OF(omove)(p, &ixy, mv);
            for (; OF(onormal_error)(p, &ixy) < ww; OF(oadvance)(p, &ixy)) {
                OF(ovisit)(p, &ixy, s);
                for (int j = 1; j < 3; j++) {
                    int aj = (ax + j) % 3;
                    if (!ixy.next[aj]) continue;
                    OF(oiter) ix = OF(ocollapse)(p, &ixy, aj);
                    for (OF(oadvance)(p, &ix); OF(onormal_error)(p, &ix) < ww; OF(oadvance)(p, &ix))
                        OF(ovisit)(p, &ix, s);
                }
            }
        }
    }
}

/* walk one line and hand every drawn pixel (error <= 1, inside the frame) to the sink */
static void OF(odraw_line)(const OT *ln, int n, const OF(osink) *s)
{
    OF(oplot) p;
    OF(oiter) it;
    if (!OF(oplot_init)(&p, ln, n, &it)) return;
    if (n == 2) OF(odraw_2d)(&p, it, s);
    else OF(odraw_3d)(&p, it, s);
}

/* ---- draw_lines ------------------------------------------------------------------ */

typedef struct { int64_t flat; int64_t frame; OT value; } OF(orec);

typedef struct {
    OF(orec) *data;
    size_t size, cap;
    int failed;
} OF(obuf);

static void OF(obuf_push)(OF(obuf) *b, int64_t flat, int64_t frame, OT v)
{
    if (b->failed) return;
    if (b->size == b->cap) {
        size_t nc = b->cap ? 2 * b->cap : 4096;
        OF(orec) *nd = (OF(orec) *)realloc(b->data, nc * sizeof(OF(orec)));
        if (!nd) { b->failed = 1; return; }
        b->data = nd; b->cap = nc;
    }
    b->data[b->size].flat = flat;
    b->data[b->size].frame = frame;
    b->data[b->size].value = v;
    b->size++;
}

typedef struct {
    OF(obuf) *buf;
    int64_t frame;
    OT max_val;
    int kernel;
} OF(odraw_ctx);

static void OF(odraw_emit)(void *vctx, int64_t flat, OT err)
{
    OF(odraw_ctx) *c = (OF(odraw_ctx) *)vctx;
    OT v = c->max_val * OF(oprofile)(c->kernel, (OT)sqrt(err));
    OF(obuf_push)(c->buf, flat, c->frame, v);
}

/* draw_lines_nd_impl (bresenham.cpp:38-101).  Each thread walks a contiguous block of
 * lines into its own buffer; buffers are then merged into `out` (in thread order when
 * num_threads == 1, which reproduces the reference's single-thread accumulation order
 * exactly; in completion order otherwise, like the reference's omp critical). */
int OF(cbc_oracle_draw_lines)(OT *out, int64_t n_frames, int ndim, const int64_t *shape,
                              const OT *lines, int64_t n_lines, const int64_t *idxs,
                              OT max_val, int kernel, int overlap, int num_threads)
{
    if (ndim != 2 && ndim != 3) return 1;
    if (kernel < 0 || kernel > 4 || overlap < 0 || overlap > 1) return 1;
    if (n_lines < 0 || n_frames < 0) return 1;
    int64_t fsize = 1;
    for (int i = 0; i < ndim; i++) fsize *= shape[i];
    int L = 2 * ndim + 1;
    /* fill_indices / check_indices */
    int64_t *own = NULL;
    if (!idxs && n_lines) {
        own = (int64_t *)malloc(sizeof(int64_t) * (size_t)n_lines);
        if (!own) return 1;
        if (n_frames == 1) { for (int64_t i = 0; i < n_lines; i++) own[i] = 0; }
        else if (n_frames == n_lines) { for (int64_t i = 0; i < n_lines; i++) own[i] = i; }
        else { free(own); return 1; }
        idxs = own;
    } else if (n_lines) {
        for (int64_t i = 0; i < n_lines; i++)
            if (idxs[i] < 0 || idxs[i] >= n_frames) return 2;
    }
    if (num_threads < 1) num_threads = 1;
    int rc = 0;
#pragma omp parallel num_threads(num_threads)
    {
        OF(obuf) buf = {NULL, 0, 0, 0};
        OF(odraw_ctx) ctx = {&buf, 0, max_val, kernel};
        OF(osink) sink = {ndim, shape, (OT)0, OF(odraw_emit), &ctx};
#pragma omp for schedule(static) nowait
        for (int64_t i = 0; i < n_lines; i++) {
            ctx.frame = idxs[i];
            sink.width = lines[L * i + 2 * ndim];
            OF(odraw_line)(lines + L * i, ndim, &sink);
        }
#pragma omp critical
        {
            if (buf.failed) rc = 1;
            for (size_t k = 0; k < buf.size; k++) {
                int64_t index = buf.data[k].flat + fsize * buf.data[k].frame;
                OT v = buf.data[k].value;
                if (overlap) out[index] = OF(omax)(out[index], v);
                else out[index] = out[index] + v;
            }
        }
        free(buf.data);
    }
    free(own);
    return rc;
}

/* ---- accumulate_lines ------------------------------------------------------------ */

typedef struct {
    OT *scratch;          /* one frame, zero outside the current term */
    int64_t *touched;     /* flat indices written in the current term */
    size_t ntouched, cap;
    int failed;
    OT max_val;
    int kernel;
    int term_max;
} OF(oacc_ctx);

static void OF(oacc_emit)(void *vctx, int64_t flat, OT err)
{
    OF(oacc_ctx) *c = (OF(oacc_ctx) *)vctx;
    if (c->failed) return;
    OT v = c->max_val * OF(oprofile)(c->kernel, (OT)sqrt(err));
    if (c->scratch[flat] == (OT)0) {
        if (c->ntouched == c->cap) {
            size_t nc = c->cap ? 2 * c->cap : 4096;
            int64_t *nd = (int64_t *)realloc(c->touched, nc * sizeof(int64_t));
            if (!nd) { c->failed = 1; return; }
            c->touched = nd; c->cap = nc;
        }
        c->touched[c->ntouched++] = flat;
    }
    if (c->term_max) c->scratch[flat] = OF(omax)(c->scratch[flat], v);
    else c->scratch[flat] = c->scratch[flat] + v;
}

static int64_t *OF(osort_terms_keys);
static int OF(oterm_cmp)(const void *a, const void *b)
{
    int64_t ia = *(const int64_t *)a, ib = *(const int64_t *)b;
    int64_t ta = OF(osort_terms_keys)[ia], tb = OF(osort_terms_keys)[ib];
    if (ta != tb) return ta < tb ? -1 : 1;
    return ia < ib ? -1 : (ia > ib);
}

/* accumulate_lines_nd_impl (bresenham.cpp:151-259): lines grouped by term (stable in
 * line order), each term rendered into a scratch frame with in_overlap, then combined
 * into frame frames[term] of `out` with out_overlap.  Like the reference, the terms are
 * shared out among num_threads threads (bresenham.cpp:200-206), each with its own
 * scratch frame; a term's merge into `out` runs in a critical section.  With one
 * thread the terms run in ascending order. */
int OF(cbc_oracle_accumulate_lines)(OT *out, int64_t n_frames, int ndim, const int64_t *shape,
                                    const OT *lines, int64_t n_lines, const int64_t *terms,
                                    const int64_t *frames, int64_t n_terms, OT max_val,
                                    int kernel, int in_overlap, int out_overlap, int num_threads)
{
    if (ndim != 2 && ndim != 3) return 1;
    if (kernel < 0 || kernel > 4) return 1;
    if (in_overlap < 0 || in_overlap > 1 || out_overlap < 0 || out_overlap > 1) return 1;
    int64_t fsize = 1;
    for (int i = 0; i < ndim; i++) fsize *= shape[i];
    int L = 2 * ndim + 1;
    for (int64_t t = 0; t < n_terms; t++) if (frames[t] < 0 || frames[t] >= n_frames) return 2;
    for (int64_t i = 0; i < n_lines; i++) if (terms[i] < 0 || terms[i] >= n_terms) return 2;
    int64_t *order = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n_lines ? n_lines : 1));
    int64_t *offs = (int64_t *)calloc((size_t)n_terms + 1, sizeof(int64_t));
    if (!order || !offs) { free(order); free(offs); return 1; }
    for (int64_t i = 0; i < n_lines; i++) order[i] = i;
    OF(osort_terms_keys) = (int64_t *)terms;
    qsort(order, (size_t)n_lines, sizeof(int64_t), OF(oterm_cmp));
    for (int64_t i = 0; i < n_lines; i++) offs[terms[i] + 1]++;
    for (int64_t t = 0; t < n_terms; t++) offs[t + 1] += offs[t];
    int rc = 0;
    if (num_threads < 1) num_threads = 1;
#pragma omp parallel num_threads(num_threads)
    {
        OF(oacc_ctx) c = {NULL, NULL, 0, 0, 0, max_val, kernel, in_overlap};
        c.scratch = (OT *)calloc((size_t)(fsize ? fsize : 1), sizeof(OT));
        if (!c.scratch) c.failed = 1;
        OF(osink) sink = {ndim, shape, (OT)0, OF(oacc_emit), &c};
#pragma omp for schedule(dynamic, 1)
        for (int64_t t = 0; t < n_terms; t++) {
            if (c.failed) continue;
            for (int64_t k = offs[t]; k < offs[t + 1]; k++) {
                int64_t i = order[k];
                sink.width = lines[L * i + 2 * ndim];
                OF(odraw_line)(lines + L * i, ndim, &sink);
            }
            OT *dst = out + frames[t] * fsize;
#pragma omp critical(oracle_accumulate_merge)
            for (size_t k = 0; k < c.ntouched; k++) {
                int64_t f = c.touched[k];
                if (out_overlap) dst[f] = OF(omax)(dst[f], c.scratch[f]);
                else dst[f] = c.scratch[f] + dst[f];
                c.scratch[f] = (OT)0;
            }
            c.ntouched = 0;
        }
#pragma omp critical(oracle_accumulate_rc)
        if (c.failed) rc = 1;
        free(c.scratch);
        free(c.touched);
    }
    free(order); free(offs);
    return rc;
}

#undef OF
#undef OCAT
#undef OCAT2
