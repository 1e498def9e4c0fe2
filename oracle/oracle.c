/*
 * oracle.c -- CPU restatement of the reference's join semantics.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the library links or calls this file;
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm use it,
 * as the parity reference of the GPU results and the timed CPU baseline.
 *
 * Every function restates one reference algorithm (paths relative to the
 * VIDA-NYU/raster-join tree) in plain C with fp32 arithmetic evaluated one
 * operation at a time (built with -ffp-contract=off, no fast-math):
 *
 *   orc_cpujoin          CPUJoin::execute (CPUJoin/CPUJoin.cpp:62-122) over the
 *                        grid of GridIndexF::buildGrid (CPUJoin/GridIndexF.cpp:
 *                        60-155), with its rectangle test (:404-549) as written
 *   orc_index_join       the GPU index join: index-size.glsl / create-index.glsl
 *                        MBR grid + index.glsl:339-402 per point
 *   orc_hybrid_join      hybrid.glsl:224-300 semantics: points inside the
 *                        half-open polygon bounds (rasterize :187-200), counted
 *                        by exact point-in-polygon through the grid
 *   orc_bruteforce       every polygon, fp32 crossing number (no grid)
 *   orc_bruteforce_f64   every polygon, crossing number in double (diagnostic)
 *   orc_raster_join      bounded raster join: canvas + tiles (RasterJoin.cpp:
 *                        51-78, 196-243), point pass (points.vert:138-159),
 *                        pixel-centre polygon pass (polygon.frag:12-27), and
 *                        the error-bound outline pass (line-bound.frag:51-286)
 *
 * The polygon pass decides coverage per pixel centre with an exact integer
 * edge test on 1/256-pixel snapped window coordinates (the GL rasteriser's
 * rule); the reference's triangulation is not needed for that decision.
 *
 * Pinning.  The exact joins (index, hybrid, CPUJoin, brute force) are pinned
 * by the reference's own known-answer fixture (RasterJoin/test/baseline.hpp:
 * 139-217) and agree with each other exactly on seeded and edge-adversarial
 * inputs.  Raster pixel assignment is parity unpinned against the reference:
 * it is the GL driver's rasteriser, which cannot run here; the pixel-centre
 * rule is cross-checked against GL's triangle rule on the reference's own
 * triangulation (compiled from its sources into oracle/_ref).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_FILTERS 12

enum { LOCATION = 0, UINT_T = 1, INT_T = 2, FLOAT_T = 3 };
enum { EQ = 0, LT = 1, LTE = 2, GT = 3, GTE = 4 };

typedef struct {
    int n;
    const uint32_t *col[ORC_MAX_FILTERS];
    int op[ORC_MAX_FILTERS];
    int typ[ORC_MAX_FILTERS];
    uint32_t val[ORC_MAX_FILTERS];
    uint32_t compat_mask;
    int aggr;
    int aggr_typ;
    const uint32_t *aggr_col;
} orc_filter;

static int nthreads_of(int req) {
#ifdef _OPENMP
    return req > 0 ? req : omp_get_max_threads();
#else
    (void)req;
    return 1;
#endif
}
static int thread_id(void) {
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
}

static float bits_f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* aLessThan / aGreaterThan / aEqual / validFilter, points.vert:24-114 */
static int p_less(int typ, uint32_t a, uint32_t f) {
    if (typ == UINT_T) return a < f;
    if (typ == INT_T) return (int32_t)a < (int32_t)f;
    if (typ == FLOAT_T) return bits_f(a) < bits_f(f);
    return 1;
}
static int p_greater(int typ, uint32_t a, uint32_t f) {
    if (typ == UINT_T) return a > f;
    if (typ == INT_T) return (int32_t)a > (int32_t)f;
    if (typ == FLOAT_T) return bits_f(a) > bits_f(f);
    return 1;
}
static int p_equal(int typ, uint32_t a, uint32_t f) {
    if (typ == UINT_T) return a == f;
    if (typ == INT_T) return (int32_t)a == (int32_t)f;
    if (typ == FLOAT_T) return bits_f(a) == bits_f(f);
    return 1;
}
static int p_eval(int op, int typ, uint32_t a, uint32_t f, int compat) {
    int eqx = compat ? (bits_f(f) == bits_f(a)) : p_equal(typ, a, f);
    switch (op) {
        case EQ: return p_equal(typ, a, f);
        case LT: return p_less(typ, a, f);
        case LTE: return p_less(typ, a, f) || eqx;
        case GT: return p_greater(typ, a, f);
        case GTE: return p_greater(typ, a, f) || eqx;
        default: return 0;
    }
}
static int passes(const orc_filter *f, uint64_t i) {
    for (int k = 0; k < f->n; ++k)
        if (!p_eval(f->op[k], f->typ[k], f->col[k][i], f->val[k], (int)((f->compat_mask >> k) & 1u))) return 0;
    return 1;
}
/* floatVal, points.vert:116-136 */
static float value_of(const orc_filter *f, uint64_t i) {
    if (!f->aggr) return 0.0f;
    uint32_t a = f->aggr_col[i];
    if (f->aggr_typ == UINT_T) return (float)a;
    if (f->aggr_typ == INT_T) return (float)(int32_t)a;
    if (f->aggr_typ == FLOAT_T) return bits_f(a);
    return 0.0f;
}

/* isInsidePoly, index.glsl:47-67 / GridIndexF.cpp:383-402 (fp32). */
static int pip32(const float *v, int n, float tx, float ty) {
    int c = 0;
    for (int i = 0, j = n - 1; i < n; j = i++) {
        float vix = v[2 * i], viy = v[2 * i + 1], vjx = v[2 * j], vjy = v[2 * j + 1];
        if ((viy > ty) != (vjy > ty)) {
            float a = vjx - vix;
            float b = ty - viy;
            float num = a * b;
            float den = vjy - viy;
            float q = num / den;
            float xi = q + vix;
            if (tx < xi) c = !c;
        }
    }
    return c;
}

static int pip64(const float *v, int n, double tx, double ty) {
    int c = 0;
    for (int i = 0, j = n - 1; i < n; j = i++) {
        double vix = v[2 * i], viy = v[2 * i + 1], vjx = v[2 * j], vjy = v[2 * j + 1];
        if (((viy > ty) != (vjy > ty)) && (tx < (vjx - vix) * (ty - viy) / (vjy - viy) + vix)) c = !c;
    }
    return c;
}

/* Per-thread accumulators reduced at the end (CPUJoin.cpp:93-116). */
typedef struct {
    int P, nt;
    uint64_t *cnt;
    double *sum;
} accum;
static void acc_init(accum *a, int P, int nt) {
    a->P = P; a->nt = nt;
    a->cnt = (uint64_t *)calloc((size_t)P * nt, sizeof(uint64_t));
    a->sum = (double *)calloc((size_t)P * nt, sizeof(double));
}
static void acc_finish(accum *a, uint64_t *count, double *sum) {
    for (int p = 0; p < a->P; ++p) {
        uint64_t c = 0;
        double s = 0.0;
        for (int t = 0; t < a->nt; ++t) { c += a->cnt[(size_t)t * a->P + p]; s += a->sum[(size_t)t * a->P + p]; }
        if (count) count[p] = c;
        if (sum) sum[p] = s;
    }
    free(a->cnt);
    free(a->sum);
}

/* ------------------------------------------------------------------------- */
/* Brute force over every polygon (fp32 crossing number).  Points outside the
 * closed polygon-set bounds are skipped. */
void orc_bruteforce(const float *xy, uint64_t n, const orc_filter *f, const float *verts, const int *pindex,
                    int P, const double *bbox, int nthreads, uint64_t *count, double *sum) {
    int nt = nthreads_of(nthreads);
    float *mbr = (float *)malloc(sizeof(float) * 4 * (size_t)P);
    float ex = (float)((bbox[2] - bbox[0] + bbox[3] - bbox[1]) * 1e-3);
    for (int p = 0; p < P; ++p) {
        float a = INFINITY, b = INFINITY, c = -INFINITY, d = -INFINITY;
        for (int k = pindex[p]; k < pindex[p + 1]; ++k) {
            float x = verts[2 * k], y = verts[2 * k + 1];
            a = fminf(a, x); b = fminf(b, y); c = fmaxf(c, x); d = fmaxf(d, y);
        }
        mbr[4 * p] = a - ex; mbr[4 * p + 1] = b - ex; mbr[4 * p + 2] = c + ex; mbr[4 * p + 3] = d + ex;
    }
    accum ac;
    acc_init(&ac, P, nt);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        float x = xy[2 * i], y = xy[2 * i + 1];
        if (!(x >= bbox[0] && x <= bbox[2] && y >= bbox[1] && y <= bbox[3])) continue;
        if (!passes(f, (uint64_t)i)) continue;
        float v = value_of(f, (uint64_t)i);
        int th = thread_id();
        for (int p = 0; p < P; ++p) {
            if (x < mbr[4 * p] || x > mbr[4 * p + 2] || y < mbr[4 * p + 1] || y > mbr[4 * p + 3]) continue;
            int v0 = pindex[p], nv = pindex[p + 1] - v0;
            if (nv > 0 && pip32(verts + 2 * v0, nv, x, y)) {
                ac.cnt[(size_t)th * P + p]++;
                ac.sum[(size_t)th * P + p] += (double)v;
            }
        }
    }
    acc_finish(&ac, count, sum);
    free(mbr);
}

/* Brute force in double precision (reference-independent diagnostic). */
void orc_bruteforce_f64(const float *xy, uint64_t n, const orc_filter *f, const float *verts, const int *pindex,
                        int P, int nthreads, uint64_t *count, double *sum) {
    int nt = nthreads_of(nthreads);
    accum ac;
    acc_init(&ac, P, nt);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        if (!passes(f, (uint64_t)i)) continue;
        double x = xy[2 * i], y = xy[2 * i + 1];
        double v = (double)value_of(f, (uint64_t)i);
        int th = thread_id();
        for (int p = 0; p < P; ++p) {
            int v0 = pindex[p], nv = pindex[p + 1] - v0;
            if (nv > 0 && pip64(verts + 2 * v0, nv, x, y)) {
                ac.cnt[(size_t)th * P + p]++;
                ac.sum[(size_t)th * P + p] += v;
            }
        }
    }
    acc_finish(&ac, count, sum);
}

/* ------------------------------------------------------------------------- */
/* GPU index join semantics.  Grid over the polygon bounds: lower-left and cell
 * size as fp32 uniforms (GLFunction.cpp:207-209); per polygon the MBR cells
 * [int((min-lb)/cs), int((max-lb)/cs)+1) with the upper bound clamped to res
 * (default) or res-1 (compat=1, create-index.glsl:56-61); per point the cell
 * int((p-lb)/cs) (index.glsl:382-385), then every listed polygon's fp32
 * crossing-number test. */
typedef struct {
    int res;
    float lbx, lby, csx, csy;
    int *start;   /* res*res + 1 */
    int *entries;
} orc_grid;

static void grid_build_mbr(orc_grid *g, const float *verts, const int *pindex, int P, const double *bbox, int res,
                           int compat) {
    double dx = bbox[2] - bbox[0], dy = bbox[3] - bbox[1];
    g->res = res;
    g->lbx = (float)bbox[0];
    g->lby = (float)bbox[1];
    g->csx = (float)(dx / res);
    g->csy = (float)(dy / res);
    size_t nc = (size_t)res * res;
    int *cnt = (int *)calloc(nc, sizeof(int));
    int *rng = (int *)malloc(sizeof(int) * 4 * (size_t)P);
    for (int p = 0; p < P; ++p) {
        int v0 = pindex[p], nv = pindex[p + 1] - v0;
        float lbx = INFINITY, lby = INFINITY, rtx = -INFINITY, rty = -INFINITY;
        for (int k = 0; k < nv; ++k) {
            float x = verts[2 * (v0 + k)], y = verts[2 * (v0 + k) + 1];
            lbx = fminf(lbx, x); rtx = fmaxf(rtx, x); lby = fminf(lby, y); rty = fmaxf(rty, y);
        }
        float qx0 = (lbx - g->lbx) / g->csx, qy0 = (lby - g->lby) / g->csy;
        float qx1 = (rtx - g->lbx) / g->csx, qy1 = (rty - g->lby) / g->csy;
        int stx = (int)qx0, sty = (int)qy0, enx = (int)qx1 + 1, eny = (int)qy1 + 1;
        int cap = compat ? res - 1 : res;
        if (enx >= cap) enx = cap;
        if (eny >= cap) eny = cap;
        if (stx < 0) stx = 0;
        if (sty < 0) sty = 0;
        if (nv == 0) { enx = stx; eny = sty; }
        rng[4 * p] = stx; rng[4 * p + 1] = sty; rng[4 * p + 2] = enx; rng[4 * p + 3] = eny;
        for (int y = sty; y < eny; ++y)
            for (int x = stx; x < enx; ++x) cnt[(size_t)y * res + x]++;
    }
    g->start = (int *)malloc(sizeof(int) * (nc + 1));
    g->start[0] = 0;
    for (size_t c = 0; c < nc; ++c) g->start[c + 1] = g->start[c] + cnt[c];
    g->entries = (int *)malloc(sizeof(int) * ((size_t)g->start[nc] + 1));
    memset(cnt, 0, nc * sizeof(int));
    for (int p = 0; p < P; ++p)
        for (int y = rng[4 * p + 1]; y < rng[4 * p + 3]; ++y)
            for (int x = rng[4 * p]; x < rng[4 * p + 2]; ++x) {
                size_t c = (size_t)y * res + x;
                g->entries[g->start[c] + cnt[c]++] = p;
            }
    free(cnt);
    free(rng);
}

static int grid_cell(const orc_grid *g, float x, float y) {
    float qx = (x - g->lbx) / g->csx;
    float qy = (y - g->lby) / g->csy;
    if (!(qx > -1.0f && qx < (float)g->res && qy > -1.0f && qy < (float)g->res)) return -1;
    return (int)qx + g->res * (int)qy;
}

/* hybrid.glsl rasterize() validity: half-open [-1,1) in fp32 (:187-200). */
static int hyb_inside(const double *bbox, float x, float y) {
    float lbx = (float)bbox[0], lby = (float)bbox[1], rtx = (float)bbox[2], rty = (float)bbox[3];
    float sx = rtx + lbx, sy = rty + lby, qx = rtx - lbx, qy = rty - lby;
    float ox = sx / 2.0f, oy = sy / 2.0f, dx = qx / 2.0f, dy = qy / 2.0f;
    float u = (x - ox) / dx, v = (y - oy) / dy;
    return !(u < -1.0f || u >= 1.0f || v < -1.0f || v >= 1.0f);
}

static void index_like(const float *xy, uint64_t n, const orc_filter *f, const float *verts, const int *pindex,
                       int P, const double *bbox, int res, int compat, int hybrid, int nthreads, uint64_t *count,
                       double *sum) {
    int nt = nthreads_of(nthreads);
    orc_grid g;
    grid_build_mbr(&g, verts, pindex, P, bbox, res, compat);
    accum ac;
    acc_init(&ac, P, nt);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        float x = xy[2 * i], y = xy[2 * i + 1];
        if (hybrid && !hyb_inside(bbox, x, y)) continue;
        if (!passes(f, (uint64_t)i)) continue;
        int c = grid_cell(&g, x, y);
        if (c < 0) continue;
        float v = value_of(f, (uint64_t)i);
        int th = thread_id();
        for (int k = g.start[c]; k < g.start[c + 1]; ++k) {
            int p = g.entries[k];
            int v0 = pindex[p], nv = pindex[p + 1] - v0;
            if (nv > 0 && pip32(verts + 2 * v0, nv, x, y)) {
                ac.cnt[(size_t)th * P + p]++;
                ac.sum[(size_t)th * P + p] += (double)v;
            }
        }
    }
    acc_finish(&ac, count, sum);
    free(g.start);
    free(g.entries);
}

void orc_index_join(const float *xy, uint64_t n, const orc_filter *f, const float *verts, const int *pindex, int P,
                    const double *bbox, int res, int compat, int nthreads, uint64_t *count, double *sum) {
    index_like(xy, n, f, verts, pindex, P, bbox, res, compat, 0, nthreads, count, sum);
}

void orc_hybrid_join(const float *xy, uint64_t n, const orc_filter *f, const float *verts, const int *pindex, int P,
                     const double *bbox, int res, int nthreads, uint64_t *count, double *sum) {
    index_like(xy, n, f, verts, pindex, P, bbox, res, 0, 1, nthreads, count, sum);
}

/* ------------------------------------------------------------------------- */
/* CPUJoin restatement (count only, as the reference; filters/avg optional as
 * a labelled extension).  GridIndexF: width/height in fp32 (:66-67), getXIndex
 * (:39-47), buildGrid inclusive loops with the rectangle test (:83-125),
 * getRegion (:158-175). */
#define OC_INSIDE 0
#define OC_LEFT 1
#define OC_RIGHT 2
#define OC_BOTTOM 4
#define OC_TOP 8

static int cs_outcode_cpu(float x, float y, float lbx, float lby, float rtx, float rty) {
    int code = OC_INSIDE;
    if (x < lbx) code |= OC_LEFT;
    else if (x > rtx) code |= OC_RIGHT;
    if (y < lby) code |= OC_BOTTOM;
    else if (y > rty) code |= OC_TOP;
    return code;
}

/* GridIndexF::rayToLineSegmentIntersection :513-549 */
static int ray_seg(float ox, float oy, float dxr, float dyr, float p0x, float p0y, float p1x, float p1y, float *rx,
                   float *ry) {
    float x1 = ox, y1 = oy;
    float x2 = ox + dxr, y2 = oy + dyr;
    float x3 = p0x, y3 = p0y, x4 = p1x, y4 = p1y;
    float s1 = (y2 - y1) / (x2 - x1);
    float s2 = (y4 - y3) / (x4 - x3);
    if (s1 != s2) {
        float d = ((x2 - x1) * (y4 - y3)) - (y2 - y1) * (x4 - x3);
        if (d != 0) {
            float r = (((y1 - y3) * (x4 - x3)) - (x1 - x3) * (y4 - y3)) / d;
            float s = (((y1 - y3) * (x2 - x1)) - (x1 - x3) * (y2 - y1)) / d;
            if (r >= 0) {
                if (s >= 0 && s <= 1) {
                    float mx = dxr * r, my = dyr * r;
                    *rx = ox + mx;
                    *ry = oy + my;
                    return 1;
                }
            }
        }
    }
    return 0;
}

/* GridIndexF::lineRectIntersection :404-424, including the second test's
 * comparison of res.y() against rightTop.x() (:412). */
static int line_rect(float v1x, float v1y, float v2x, float v2y, float lbx, float lby, float rtx, float rty) {
    float rx, ry;
    if (ray_seg(lbx, lby, 0.0f, 1.0f, v1x, v1y, v2x, v2y, &rx, &ry) && ry <= rty) return 1;
    if (ray_seg(lbx, lby, 1.0f, 0.0f, v1x, v1y, v2x, v2y, &rx, &ry) && ry <= rtx) return 1;
    if (ray_seg(rtx, rty, 0.0f, -1.0f, v1x, v1y, v2x, v2y, &rx, &ry) && ry >= lby) return 1;
    if (ray_seg(rtx, rty, -1.0f, 0.0f, v1x, v1y, v2x, v2y, &rx, &ry) && rx >= lbx) return 1;
    return 0;
}

/* GridIndexF::polygonRectIntersectionCPU :461-496 (the closing edge is not
 * tested in case 3, as written). */
static int poly_rect(const float *v, int n, float lbx, float lby, float rtx, float rty) {
    for (int i = 0; i < n; ++i) {
        float x = v[2 * i], y = v[2 * i + 1];
        if (x >= lbx && x <= rtx && y >= lby && y <= rty) return 1;
    }
    if (pip32(v, n, lbx, lby)) return 1;
    if (pip32(v, n, rtx, rty)) return 1;
    if (pip32(v, n, lbx, rty)) return 1;
    if (pip32(v, n, rtx, lby)) return 1;
    int c2 = cs_outcode_cpu(v[0], v[1], lbx, lby, rtx, rty);
    for (int i = 0; i < n - 1; ++i) {
        int c1 = c2;
        c2 = cs_outcode_cpu(v[2 * (i + 1)], v[2 * (i + 1) + 1], lbx, lby, rtx, rty);
        if (!(c1 & c2) && line_rect(v[2 * i], v[2 * i + 1], v[2 * (i + 1)], v[2 * (i + 1) + 1], lbx, lby, rtx, rty))
            return 1;
    }
    return 0;
}

typedef struct {
    int xs, ys;
    float minx, miny, width, height;
    int *start;
    int *entries;
} orc_cpugrid;

static void cpugrid_build(orc_cpugrid *g, const float *verts, const int *pindex, int P, const double *bbox, int res,
                          int nthreads) {
    int nt = nthreads_of(nthreads);
    g->xs = g->ys = res;
    float minx = (float)bbox[0], miny = (float)bbox[1], maxx = (float)bbox[2], maxy = (float)bbox[3];
    g->minx = minx;
    g->miny = miny;
    g->width = (maxx - minx) / res;
    g->height = (maxy - miny) / res;
    size_t nc = (size_t)res * res;
    /* per polygon candidate lists, then CSR by cell in polygon order */
    int **lists = (int **)calloc((size_t)P, sizeof(int *));
    int *nlist = (int *)calloc((size_t)P, sizeof(int));
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
    for (int p = 0; p < P; ++p) {
        int v0 = pindex[p], nv = pindex[p + 1] - v0;
        const float *pv = verts + 2 * v0;
        float bminx = INFINITY, bminy = INFINITY, bmaxx = -INFINITY, bmaxy = -INFINITY;
        for (int k = 0; k < nv; ++k) {
            bminx = fminf(bminx, pv[2 * k]); bmaxx = fmaxf(bmaxx, pv[2 * k]);
            bminy = fminf(bminy, pv[2 * k + 1]); bmaxy = fmaxf(bmaxy, pv[2 * k + 1]);
        }
        if (nv == 0) continue;
        int stx = (int)((bminx - minx) / g->width);
        int enx = (int)((bmaxx - minx) / g->width) + 1;
        int sty = (int)((bminy - miny) / g->height);
        int eny = (int)((bmaxy - miny) / g->height) + 1;
        if (enx >= res) enx = res - 1;
        if (eny >= res) eny = res - 1;
        if (stx < 0) stx = 0;
        if (sty < 0) sty = 0;
        int cap = 64, m = 0;
        int *l = (int *)malloc(sizeof(int) * cap);
        for (int x = stx; x <= enx; ++x) {
            for (int y = sty; y <= eny; ++y) {
                float lbx = x * g->width + minx, lby = y * g->height + miny;
                float rtx = (x + 1) * g->width + minx, rty = (y + 1) * g->height + miny;
                if (poly_rect(pv, nv, lbx, lby, rtx, rty)) {
                    if (m == cap) { cap *= 2; l = (int *)realloc(l, sizeof(int) * cap); }
                    l[m++] = y * res + x;
                }
            }
        }
        lists[p] = l;
        nlist[p] = m;
    }
    int *cnt = (int *)calloc(nc, sizeof(int));
    for (int p = 0; p < P; ++p)
        for (int k = 0; k < nlist[p]; ++k) cnt[lists[p][k]]++;
    g->start = (int *)malloc(sizeof(int) * (nc + 1));
    g->start[0] = 0;
    for (size_t c = 0; c < nc; ++c) g->start[c + 1] = g->start[c] + cnt[c];
    g->entries = (int *)malloc(sizeof(int) * ((size_t)g->start[nc] + 1));
    memset(cnt, 0, nc * sizeof(int));
    for (int p = 0; p < P; ++p) {
        for (int k = 0; k < nlist[p]; ++k) {
            int c = lists[p][k];
            g->entries[g->start[c] + cnt[c]++] = p;
        }
        free(lists[p]);
    }
    free(lists);
    free(nlist);
    free(cnt);
}

static void cpugrid_free(orc_cpugrid *g) {
    free(g->start);
    free(g->entries);
}

/* Grid build time is reported separately, as CPUJoin.cpp:124-163 does. */
double orc_cpujoin(const float *xy, uint64_t n, const orc_filter *f, const float *verts, const int *pindex, int P,
                   const double *bbox, int res, int nthreads, uint64_t *count, double *sum, double *build_seconds) {
    int nt = nthreads_of(nthreads);
    double t0 = 0, t1 = 0;
#ifdef _OPENMP
    t0 = omp_get_wtime();
#endif
    orc_cpugrid g;
    cpugrid_build(&g, verts, pindex, P, bbox, res, nt);
#ifdef _OPENMP
    t1 = omp_get_wtime();
#endif
    if (build_seconds) *build_seconds = t1 - t0;
    accum ac;
    acc_init(&ac, P, nt);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        float x = xy[2 * i], y = xy[2 * i + 1];
        if (f && !passes(f, (uint64_t)i)) continue;
        int stx = (int)((x - g.minx) / g.width);
        int sty = (int)((y - g.miny) / g.height);
        float qx = (x - g.minx) / g.width, qy = (y - g.miny) / g.height;
        if (!(qx > -1.0f && qx < (float)res && qy > -1.0f && qy < (float)res)) continue;
        if (stx < 0 || stx >= g.xs || sty < 0 || sty >= g.ys) continue;
        int c = sty * res + stx;
        float v = f ? value_of(f, (uint64_t)i) : 0.0f;
        int th = thread_id();
        for (int k = g.start[c]; k < g.start[c + 1]; ++k) {
            int p = g.entries[k];
            int v0 = pindex[p], nv = pindex[p + 1] - v0;
            if (pip32(verts + 2 * v0, nv, x, y)) {
                ac.cnt[(size_t)th * P + p]++;
                ac.sum[(size_t)th * P + p] += (double)v;
            }
        }
    }
    acc_finish(&ac, count, sum);
    cpugrid_free(&g);
    double t2 = t1;
#ifdef _OPENMP
    t2 = omp_get_wtime();
#endif
    return t2 - t1;
}

/* ------------------------------------------------------------------------- */
/* Bounded raster join. */
#define SUB 256

/* One axis of the tile grid: RasterJoin::updateBuffers + getMVP. */
typedef struct {
    int split, res;
    float *s, *t, h;
} orc_axis;

static void axis_plan(orc_axis *a, double lo, double hi, double cell, int max_res) {
    double d = hi - lo;
    int actual = (int)ceil(d / cell);
    if (actual < 1) actual = 1;
    a->split = (int)ceil((double)actual / max_res);
    a->res = (int)ceil((double)actual / a->split);
    a->s = (float *)malloc(sizeof(float) * a->split);
    a->t = (float *)malloc(sizeof(float) * a->split);
    double td = d / a->split;
    for (int c = 0; c < a->split; ++c) {
        double lb = lo + c * td, rt = lb + td;
        double origin = (rt + lb) / 2, half = (rt - lb) / 2;
        float s = (float)(1.0 / half);
        float mo = (float)(-origin);
        float t = s * mo;
        a->s[c] = s;
        a->t[c] = t;
    }
    a->h = a->res * 0.5f;
}
static void axis_free(orc_axis *a) { free(a->s); free(a->t); }

static float win(float v, float s, float t, float h) {
    float p = s * v;
    float ndc = p + t;
    float q = h * ndc;
    return q + h;
}
static int32_t snapw(float w) {
    if (w < -1048576.0f) w = -1048576.0f;
    if (w > 1048576.0f) w = 1048576.0f;
    float z = w * 256.0f;
    return (int32_t)lrintf(z);
}
static int32_t floor256(int32_t X) {
    int32_t q = X / SUB;
    if ((X % SUB) != 0 && X < 0) --q;
    return q;
}
/* exact: does edge (A,B) toggle the pixel centre (cx,cy)?  Half-open in y
 * ((A.y >= cy) != (B.y >= cy)) and strictly left of the crossing in x. */
static int edge_toggles_exact(int64_t ax, int64_t ay, int64_t bx, int64_t by, int64_t cx, int64_t cy) {
    if ((ay >= cy) == (by >= cy)) return 0;
    int64_t dy = by - ay;
    int64_t lhs = (cx - ax) * dy;
    int64_t rhs = (bx - ax) * (cy - ay);
    return dy > 0 ? (lhs < rhs) : (lhs > rhs);
}
static int covers(const int32_t *wx, const int32_t *wy, int n, int i, int j) {
    int64_t cx = (int64_t)i * SUB + SUB / 2, cy = (int64_t)j * SUB + SUB / 2;
    int c = 0;
    for (int k = 0; k < n; ++k) {
        int kn = (k + 1 == n) ? 0 : k + 1;
        c ^= edge_toggles_exact(wx[k], wy[k], wx[kn], wy[kn], cx, cy);
    }
    return c;
}

/* computeFraction, line-bound.frag:51-211, in window units. */
static int cs_code(float x, float y, float xmin, float ymin, float xmax, float ymax) {
    int code = 0;
    if (x < xmin) code |= 1;
    else if (x > xmax) code |= 2;
    if (y < ymin) code |= 4;
    else if (y > ymax) code |= 8;
    return code;
}
static float tri_area(float ax, float ay, float bx, float by, float cx, float cy) {
    float ix = bx - ax, iy = by - ay, jx = cx - ax, jy = cy - ay;
    float p1 = ix * jy, p2 = iy * jx;
    float cz = p1 - p2;
    float h = 0.5f * cz;
    return fabsf(h);
}
static int compute_fraction(float x0, float y0, float x1, float y1, float xmin, float ymin, float xmax, float ymax,
                            float *frac) {
    int oc0 = cs_code(x0, y0, xmin, ymin, xmax, ymax), oc1 = cs_code(x1, y1, xmin, ymin, xmax, ymax);
    int accept = 0;
    *frac = 0.0f;
    for (int it = 0; it < 16; ++it) {
        if ((oc0 | oc1) == 0) { accept = 1; break; }
        if ((oc0 & oc1) != 0) break;
        float x = 0.0f, y = 0.0f;
        int out = oc0 ? oc0 : oc1;
        if (out & 8) { float a = x1 - x0, b = ymax - y0, m = a * b, d = y1 - y0, q = m / d; x = x0 + q; y = ymax; }
        else if (out & 4) { float a = x1 - x0, b = ymin - y0, m = a * b, d = y1 - y0, q = m / d; x = x0 + q; y = ymin; }
        else if (out & 2) { float a = y1 - y0, b = xmax - x0, m = a * b, d = x1 - x0, q = m / d; y = y0 + q; x = xmax; }
        else if (out & 1) { float a = y1 - y0, b = xmin - x0, m = a * b, d = x1 - x0, q = m / d; y = y0 + q; x = xmin; }
        if (out == oc0) { x0 = x; y0 = y; oc0 = cs_code(x0, y0, xmin, ymin, xmax, ymax); }
        else { x1 = x; y1 = y; oc1 = cs_code(x1, y1, xmin, ymin, xmax, ymax); }
    }
    if (!accept) return 0;
    if (x0 > x1) { float t = x0; x0 = x1; x1 = t; t = y0; y0 = y1; y1 = t; }
    float v1x = 0, v1y = 0, v2x = 0, v2y = 0, v3x = 0, v3y = 0, v4x = 0, v4y = 0;
    int tri = 0, compute = 1;
    if (x0 == xmin) {
        if (x1 == xmax) { v1x = xmin; v1y = ymin; v2x = xmax; v2y = ymin; v3x = x1; v3y = y1; v4x = x0; v4y = y0; }
        else if (y1 == ymax) { v1x = xmin; v1y = ymax; v2x = x0; v2y = y0; v3x = x1; v3y = y1; tri = 1; }
        else if (y1 == ymin) { v1x = xmin; v1y = ymin; v2x = x0; v2y = y0; v3x = x1; v3y = y1; tri = 1; }
        else compute = 0;
    } else if (x1 == xmax) {
        if (y0 == ymax) { v1x = xmax; v1y = ymax; v2x = x0; v2y = y0; v3x = x1; v3y = y1; tri = 1; }
        else if (y0 == ymin) { v1x = xmax; v1y = ymin; v2x = x1; v2y = y1; v3x = x0; v3y = y0; tri = 1; }
        else compute = 0;
    } else if (y0 == ymin && y1 == ymax) {
        v1x = xmin; v1y = ymin; v2x = xmin; v2y = ymax; v3x = x1; v3y = y1; v4x = x0; v4y = y0;
    } else if (y1 == ymin && y0 == ymax) {
        v1x = xmin; v1y = ymin; v2x = xmin; v2y = ymax; v3x = x0; v3y = y0; v4x = x1; v4y = y1;
    } else compute = 0;
    *frac = 0.5f;
    if (compute) {
        float area = tri_area(v1x, v1y, v2x, v2y, v3x, v3y);
        if (!tri) area = area + tri_area(v1x, v1y, v3x, v3y, v4x, v4y);
        float den = (ymax - ymin) * (xmax - xmin);
        *frac = area / den;
    }
    return 1;
}

/* Outputs: count/sum per polygon; bounds (may be NULL) int64[4P]
 * [fn | fp | fn1 | fp1]; canvas_out (may be NULL) receives tile 0's counts. */
int orc_raster_join(const float *xy, uint64_t n, const orc_filter *f, const float *verts, const int *pindex, int P,
                    const double *bbox, double cell, int max_res, int line_filter, int nthreads, uint64_t *count,
                    double *sum, int64_t *bounds) {
    int nt = nthreads_of(nthreads);
    orc_axis ax, ay;
    axis_plan(&ax, bbox[0], bbox[2], cell, max_res);
    axis_plan(&ay, bbox[1], bbox[3], cell, max_res);
    const int T = ax.split * ay.split;
    const size_t tile_px = (size_t)ax.res * ay.res;
    uint32_t *cc = (uint32_t *)calloc(tile_px * T, sizeof(uint32_t));
    double *cs = f->aggr ? (double *)calloc(tile_px * T, sizeof(double)) : NULL;
    if (!cc || (f->aggr && !cs)) { free(cc); free(cs); axis_free(&ax); axis_free(&ay); return -2; }
    /* point pass: every point against every tile (RasterJoin.cpp:224-231) */
    for (uint64_t i = 0; i < n; ++i) {
        if (!passes(f, i)) continue;
        float x = xy[2 * i], y = xy[2 * i + 1];
        float v = value_of(f, i);
        for (int cx = 0; cx < ax.split; ++cx) {
            float wx = win(x, ax.s[cx], ax.t[cx], ax.h);
            if (!(wx > -1.0f && wx < (float)ax.res + 1.0f)) continue;
            int px = floor256(snapw(wx));
            if (px < 0 || px >= ax.res) continue;
            for (int cy = 0; cy < ay.split; ++cy) {
                float wy = win(y, ay.s[cy], ay.t[cy], ay.h);
                if (!(wy > -1.0f && wy < (float)ay.res + 1.0f)) continue;
                int py = floor256(snapw(wy));
                if (py < 0 || py >= ay.res) continue;
                size_t pix = (size_t)(cy * ax.split + cx) * tile_px + (size_t)py * ax.res + px;
                cc[pix]++;
                if (cs) cs[pix] += (double)v;
            }
        }
    }
    /* polygon pass */
    const int V = pindex[P];
    int32_t *wxs = (int32_t *)malloc(sizeof(int32_t) * (size_t)V * T);
    int32_t *wys = (int32_t *)malloc(sizeof(int32_t) * (size_t)V * T);
    float *fxs = (float *)malloc(sizeof(float) * (size_t)V * T);
    float *fys = (float *)malloc(sizeof(float) * (size_t)V * T);
    for (int t = 0; t < T; ++t) {
        int cx = t % ax.split, cy = t / ax.split;
        for (int k = 0; k < V; ++k) {
            float wx = win(verts[2 * k], ax.s[cx], ax.t[cx], ax.h);
            float wy = win(verts[2 * k + 1], ay.s[cy], ay.t[cy], ay.h);
            fxs[(size_t)t * V + k] = wx;
            fys[(size_t)t * V + k] = wy;
            wxs[(size_t)t * V + k] = snapw(wx);
            wys[(size_t)t * V + k] = snapw(wy);
        }
    }
    for (int p = 0; p < P; ++p) { count[p] = 0; if (sum) sum[p] = 0.0; }
    if (bounds) memset(bounds, 0, sizeof(int64_t) * 4 * (size_t)P);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int item = 0; item < T * P; ++item) {
        int t = item / P, p = item % P;
        int v0 = pindex[p], nv = pindex[p + 1] - v0;
        if (nv < 2) continue;
        const int32_t *wx = wxs + (size_t)t * V + v0, *wy = wys + (size_t)t * V + v0;
        int32_t xmn = INT32_MAX, xmx = INT32_MIN, ymn = INT32_MAX, ymx = INT32_MIN;
        for (int k = 0; k < nv; ++k) {
            if (wx[k] < xmn) xmn = wx[k];
            if (wx[k] > xmx) xmx = wx[k];
            if (wy[k] < ymn) ymn = wy[k];
            if (wy[k] > ymx) ymx = wy[k];
        }
        int i0 = floor256(xmn) - 1, i1 = floor256(xmx) + 1, j0 = floor256(ymn) - 1, j1 = floor256(ymx) + 1;
        if (i0 < 0) i0 = 0;
        if (j0 < 0) j0 = 0;
        if (i1 > ax.res - 1) i1 = ax.res - 1;
        if (j1 > ay.res - 1) j1 = ay.res - 1;
        uint64_t c = 0;
        double s = 0.0;
        const size_t toff = (size_t)t * tile_px;
        for (int j = j0; j <= j1; ++j)
            for (int i = i0; i <= i1; ++i)
                if (covers(wx, wy, nv, i, j)) {
                    size_t pix = toff + (size_t)j * ax.res + i;
                    c += cc[pix];
                    if (cs) s += cs[pix];
                }
        int64_t b_fn = 0, b_fp = 0, b_fn1 = 0, b_fp1 = 0;
        if (bounds) {
            const float *fx = fxs + (size_t)t * V + v0, *fy = fys + (size_t)t * V + v0;
            for (int k = 0; k < nv; ++k) {
                int kn = (k + 1 == nv) ? 0 : k + 1;
                float p0x = fx[k], p0y = fy[k], p1x = fx[kn], p1y = fy[kn];
                int ia = (int)floorf(fminf(p0x, p1x)) - 1, ib = (int)floorf(fmaxf(p0x, p1x)) + 1;
                int ja = (int)floorf(fminf(p0y, p1y)) - 1, jb = (int)floorf(fmaxf(p0y, p1y)) + 1;
                if (ia < 0) ia = 0;
                if (ja < 0) ja = 0;
                if (ib > ax.res - 1) ib = ax.res - 1;
                if (jb > ay.res - 1) jb = ay.res - 1;
                for (int j = ja; j <= jb; ++j)
                    for (int i = ia; i <= ib; ++i) {
                        uint32_t val = cc[toff + (size_t)j * ax.res + i];
                        if (val == 0) continue;
                        if (line_filter) {
                            float cxp = (float)i + 0.5f, cyp = (float)j + 0.5f;
                            float dx = p1x - p0x, dy = p1y - p0y;
                            float l2a = dx * dx, l2b = dy * dy, l2 = l2a + l2b;
                            if (!(l2 > 0.0f)) continue;
                            float ta = (cxp - p0x) * dx, tb = (cyp - p0y) * dy, tn = ta + tb;
                            float tt = tn / l2;
                            float mx = tt * dx, my = tt * dy;
                            float qx = p0x + mx, qy = p0y + my;
                            float ex = qx - cxp, ey = qy - cyp;
                            if (fabsf(ex) >= 0.5f || fabsf(ey) >= 0.5f) continue;
                        }
                        float fr;
                        if (!compute_fraction(p0x, p0y, p1x, p1y, (float)i, (float)j, (float)(i + 1), (float)(j + 1), &fr))
                            continue;
                        int inside = covers(wx, wy, nv, i, j);
                        if (fr > 0.5f) fr = 1.0f - fr;
                        float prod = fr * (float)val;
                        int toAdd = (int)ceilf(prod);
                        if (inside) { b_fp += toAdd; b_fp1 += val; }
                        else { b_fn += toAdd; b_fn1 += val; }
                    }
            }
        }
#pragma omp critical
        {
            count[p] += c;
            if (sum) sum[p] += s;
            if (bounds) {
                bounds[p] += b_fn;
                bounds[P + p] += b_fp;
                bounds[2 * P + p] += b_fn1;
                bounds[3 * P + p] += b_fp1;
            }
        }
    }
    free(wxs); free(wys); free(fxs); free(fys);
    free(cc); free(cs);
    axis_free(&ax);
    axis_free(&ay);
    return 0;
}

/* Canvas geometry as the raster join plans it, for tests. */
/* Fill-rule cross-check (single-tile canvas).  For every pixel centre:
 * poly_cover = id of the one polygon covering it by the crossing rule the
 * library implements, -1 if none, -2 if several; tri_cover = the same from
 * triangles (tri_poly[k] = polygon of triangle k) by GL's rule on the same
 * snapped window coordinates: a centre is inside a counter-clockwise triangle
 * when every edge function is positive, or zero on a left edge (going down)
 * or a top edge (horizontal, going left).  Triangle vertices pass through
 * float as the reference uploads them (PolyHandler::getTriangulation). */
int orc_cover_maps(const float *verts, const int *pindex, int P, const double *tris, const int *tri_poly, int ntri,
                   const double *bbox, double cell, int32_t *poly_cover, int32_t *tri_cover, int *dims) {
    orc_axis ax, ay;
    axis_plan(&ax, bbox[0], bbox[2], cell, 1 << 30);
    axis_plan(&ay, bbox[1], bbox[3], cell, 1 << 30);
    const int rx = ax.res, ry = ay.res;
    dims[0] = rx;
    dims[1] = ry;
    for (size_t k = 0; k < (size_t)rx * ry; ++k) { poly_cover[k] = -1; tri_cover[k] = -1; }
    const int V = pindex[P];
    int32_t *wx = (int32_t *)malloc(sizeof(int32_t) * (size_t)V), *wy = (int32_t *)malloc(sizeof(int32_t) * (size_t)V);
    for (int k = 0; k < V; ++k) {
        wx[k] = snapw(win(verts[2 * k], ax.s[0], ax.t[0], ax.h));
        wy[k] = snapw(win(verts[2 * k + 1], ay.s[0], ay.t[0], ay.h));
    }
    for (int p = 0; p < P; ++p) {
        int v0 = pindex[p], nv = pindex[p + 1] - v0;
        if (nv < 2) continue;
        for (int j = 0; j < ry; ++j)
            for (int i = 0; i < rx; ++i)
                if (covers(wx + v0, wy + v0, nv, i, j)) {
                    int32_t *c = poly_cover + (size_t)j * rx + i;
                    *c = (*c == -1) ? p : -2;
                }
    }
    for (int k = 0; k < ntri; ++k) {
        int64_t X[3], Y[3];
        for (int q = 0; q < 3; ++q) {
            X[q] = snapw(win((float)tris[6 * k + 2 * q], ax.s[0], ax.t[0], ax.h));
            Y[q] = snapw(win((float)tris[6 * k + 2 * q + 1], ay.s[0], ay.t[0], ay.h));
        }
        int64_t area = (X[1] - X[0]) * (Y[2] - Y[0]) - (X[2] - X[0]) * (Y[1] - Y[0]);
        if (area == 0) continue;
        if (area < 0) { int64_t t = X[1]; X[1] = X[2]; X[2] = t; t = Y[1]; Y[1] = Y[2]; Y[2] = t; }
        int64_t mnx = X[0], mxx = X[0], mny = Y[0], mxy = Y[0];
        for (int q = 1; q < 3; ++q) {
            if (X[q] < mnx) mnx = X[q];
            if (X[q] > mxx) mxx = X[q];
            if (Y[q] < mny) mny = Y[q];
            if (Y[q] > mxy) mxy = Y[q];
        }
        int i0 = floor256((int32_t)mnx) - 1, i1 = floor256((int32_t)mxx) + 1;
        int j0 = floor256((int32_t)mny) - 1, j1 = floor256((int32_t)mxy) + 1;
        if (i0 < 0) i0 = 0;
        if (j0 < 0) j0 = 0;
        if (i1 > rx - 1) i1 = rx - 1;
        if (j1 > ry - 1) j1 = ry - 1;
        for (int j = j0; j <= j1; ++j)
            for (int i = i0; i <= i1; ++i) {
                const int64_t cx = (int64_t)i * SUB + SUB / 2, cy = (int64_t)j * SUB + SUB / 2;
                int in = 1;
                for (int e = 0; e < 3 && in; ++e) {
                    const int64_t ax0 = X[e], ay0 = Y[e], bx0 = X[(e + 1) % 3], by0 = Y[(e + 1) % 3];
                    const int64_t f = (bx0 - ax0) * (cy - ay0) - (by0 - ay0) * (cx - ax0);
                    const int left = (by0 < ay0), top = (by0 == ay0 && bx0 < ax0);
                    if (f < 0 || (f == 0 && !(left || top))) in = 0;
                }
                if (in) {
                    int32_t *c = tri_cover + (size_t)j * rx + i;
                    const int p = tri_poly[k];
                    *c = (*c == -1 || *c == p) ? p : -2;
                }
            }
    }
    free(wx);
    free(wy);
    axis_free(&ax);
    axis_free(&ay);
    return 0;
}

void orc_raster_geometry(const double *bbox, double cell, int max_res, int *out /* splitx, splity, resx, resy */) {
    orc_axis ax, ay;
    axis_plan(&ax, bbox[0], bbox[2], cell, max_res);
    axis_plan(&ay, bbox[1], bbox[3], cell, max_res);
    out[0] = ax.split; out[1] = ay.split; out[2] = ax.res; out[3] = ay.res;
    axis_free(&ax);
    axis_free(&ay);
}
