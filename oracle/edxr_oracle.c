/* CPU oracle for the EDXRaster rasterization pipeline (test infrastructure).
 *
 * Plain-C restatement of one Renderer::RenderMesh frame
 * (EDXRaster/Core/Renderer.cpp:100-118).  Every function names the reference
 * lines it follows.  Build with -fwrapv -ffp-contract=off: integer arithmetic
 * of the reference wraps (SSE paddd/pmulld) and no float product may be fused
 * into an add.  Only tests, the smoke check and the benchmark's CPU-baseline
 * leg call this code, as the checker; the product library never links it.
 *
 * Contracts that EDXUtil (absent from the reference) would fix, restated the
 * same way in oracle/shim and in the CUDA kernels:
 *   Matrix: row-major, column vectors, components summed left to right.
 *   HomogeneousProject: invW = 1.0f/w, then x*invW, y*invW, z*invW.
 *   Snap: int(float * 16.0) with the product in double, truncation toward
 *         zero, and INT_MIN for NaN or out-of-range (x86 cvttsd2si).
 *   BoolSSE -> IntSSE: true lanes are -1.
 */
#include "edxr_oracle.h"

#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define TILE_LOG2 5 /* Tile::SIZE_LOG_2, Tile.h:12 */
#define TILE_SIZE (1 << TILE_LOG2)

static inline int wadd(int a, int b) { return (int)((uint32_t)a + (uint32_t)b); }
static inline int wsub(int a, int b) { return (int)((uint32_t)a - (uint32_t)b); }
static inline int wmul(int a, int b) { return (int)((uint32_t)a * (uint32_t)b); }
static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }

typedef struct { float x, y, z, w; } vec4f;

/* Matrix product P*MV (Renderer.cpp:90), float, k summed in order. */
static void mat_mul(const float* A, const float* B, float* C)
{
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
        {
            float s = A[i * 4 + 0] * B[0 * 4 + j];
            s = s + A[i * 4 + 1] * B[1 * 4 + j];
            s = s + A[i * 4 + 2] * B[2 * 4 + j];
            s = s + A[i * 4 + 3] * B[3 * 4 + j];
            C[i * 4 + j] = s;
        }
}

/* Matrix::TransformPoint(Vector4(p, 1)) for the vertex shader (Shader.h:45). */
static vec4f xform4(const float* M, float x, float y, float z)
{
    float o[4];
    for (int i = 0; i < 4; i++)
    {
        float s = M[i * 4 + 0] * x;
        s = s + M[i * 4 + 1] * y;
        s = s + M[i * 4 + 2] * z;
        s = s + M[i * 4 + 3] * 1.0f;
        o[i] = s;
    }
    vec4f r = { o[0], o[1], o[2], o[3] };
    return r;
}

/* Matrix::TransformPoint(Vector3) with the raster matrix
 * (RasterTriangle.h:30-32); divides only when w is not exactly 1. */
static void xform3_point(const float* M, float x, float y, float z, float out[3])
{
    float o[4];
    for (int i = 0; i < 4; i++)
    {
        float s = M[i * 4 + 0] * x;
        s = s + M[i * 4 + 1] * y;
        s = s + M[i * 4 + 2] * z;
        s = s + M[i * 4 + 3];
        o[i] = s;
    }
    if (o[3] == 1.0f)
    {
        out[0] = o[0]; out[1] = o[1]; out[2] = o[2];
    }
    else
    {
        out[0] = o[0] / o[3]; out[1] = o[1] / o[3]; out[2] = o[2] / o[3];
    }
}

/* v.x = a.x * 16.0 (RasterTriangle.h:35-40): double product, truncation. */
static int snap16(float f)
{
    const double d = (double)f * 16.0;
    if (!(d > -2147483649.0 && d < 2147483648.0))
        return INT_MIN;
    return (int)d;
}

/* ------------------------------------------------------------------------ */
/* Clipping (Clipper.h)                                                      */

enum { LEFT_BIT = 1, RIGHT_BIT = 2, BOTTOM_BIT = 4, TOP_BIT = 8, NEAR_BIT = 16, FAR_BIT = 32 };

/* Clipper::ComputeClipCode, Clipper.h:48-68 (CLIP_ALL_PLANES = 1). */
static unsigned clip_code(vec4f v)
{
    unsigned c = 0;
    if (v.x < -v.w) c |= LEFT_BIT;
    if (v.x > v.w) c |= RIGHT_BIT;
    if (v.y < -v.w) c |= BOTTOM_BIT;
    if (v.y > v.w) c |= TOP_BIT;
    if (v.z > v.w) c |= FAR_BIT;
    if (v.z < 0.0f) c |= NEAR_BIT;
    return c;
}

typedef struct { vec4f pos; float w[3]; } pvert;
/* The reference's polygon is a growable Array (Clipper.h:26); 64 slots are
 * far more than the 9 exact arithmetic allows. */
#define MAX_POLY 64
typedef struct { pvert v[MAX_POLY]; int n; } polygon;

static int plane_inside(int plane, vec4f v)
{
    switch (plane)
    {
    case 0: return v.x >= -v.w;
    case 1: return v.x <= v.w;
    case 2: return v.y >= -v.w;
    case 3: return v.y <= v.w;
    case 4: return v.z <= v.w;
    default: return v.z >= 0.0f;
    }
}

/* The t formulas of Clipper.h:241,248,255,262,269,276, written as there. */
static float plane_t(int plane, vec4f a, vec4f b)
{
    switch (plane)
    {
    case 0: return (a.w + a.x) / ((a.x + a.w) - (b.x + b.w));
    case 1: return (-a.w + a.x) / ((a.x - a.w) - (b.x - b.w));
    case 2: return (a.w + a.y) / ((a.y + a.w) - (b.y + b.w));
    case 3: return (-a.w + a.y) / ((a.y - a.w) - (b.y - b.w));
    case 4: return (-a.w + a.z) / ((a.z - a.w) - (b.z - b.w));
    default: return a.z / (a.z - b.z);
    }
}

static void plane_snap(int plane, vec4f* v)
{
    switch (plane)
    {
    case 0: v->x = -v->w; break;
    case 1: v->x = v->w; break;
    case 2: v->y = -v->w; break;
    case 3: v->y = v->w; break;
    case 4: v->z = v->w; break;
    default: v->z = 0.0f; break;
    }
}

/* Intersection vertex: pos = v0*(1-t) + v1*t, snapped onto the plane, and
 * the clip weights blended the same way (Clipper.h:210-214). */
static pvert plane_cut(int plane, const pvert* a, const pvert* b)
{
    const float t = plane_t(plane, a->pos, b->pos);
    const float s = 1 - t;
    pvert r;
    r.pos.x = a->pos.x * s + b->pos.x * t;
    r.pos.y = a->pos.y * s + b->pos.y * t;
    r.pos.z = a->pos.z * s + b->pos.z * t;
    r.pos.w = a->pos.w * s + b->pos.w * t;
    plane_snap(plane, &r.pos);
    for (int k = 0; k < 3; k++)
        r.w[k] = a->w[k] * s + b->w[k] * t;
    return r;
}

/* Clipper::ClipByPlane, Clipper.h:192-232 (Sutherland-Hodgman step). */
static void clip_by_plane(int plane, const polygon* in, polygon* out)
{
    out->n = 0;
    for (int i = 0; i < in->n; i++)
    {
        int i1 = i + 1;
        if (i1 == in->n) i1 = 0;
        const pvert* v0 = &in->v[i];
        const pvert* v1 = &in->v[i1];
        if (out->n + 2 > MAX_POLY)
            break;
        if (plane_inside(plane, v0->pos))
        {
            if (plane_inside(plane, v1->pos))
                out->v[out->n++] = *v1;
            else
                out->v[out->n++] = plane_cut(plane, v0, v1);
        }
        else if (plane_inside(plane, v1->pos))
        {
            out->v[out->n++] = plane_cut(plane, v0, v1);
            out->v[out->n++] = *v1;
        }
    }
}

/* Clipper::ClipPolygon, Clipper.h:235-288: planes L,R,B,T,F,N in that order,
 * only those in planeCode; polygons with any w <= 0 are dropped. */
static void clip_polygon(polygon* p, unsigned planeCode)
{
    static const unsigned bits[6] = { LEFT_BIT, RIGHT_BIT, BOTTOM_BIT, TOP_BIT, FAR_BIT, NEAR_BIT };
    polygon tmp;
    for (int k = 0; k < 6; k++)
    {
        if (!(planeCode & bits[k])) continue;
        clip_by_plane(k, p, &tmp);
        *p = tmp;
    }
    for (int i = 0; i < p->n; i++)
        if (p->v[i].pos.w <= 0.0f)
        {
            p->n = 0;
            return;
        }
}

/* ------------------------------------------------------------------------ */
/* Per-frame state                                                            */

/* One entry of the per-core projected-vertex buffer (Shader.h:13-25 plus the
 * per-vertex albedo of this build and the clip weights for the FP64 shade). */
typedef struct
{
    vec4f clip;   /* projectedPos as clipped; .z replaced by the post-pass */
    float invW;   /* Renderer.cpp:144 */
    float pos[3], nrm[3], uv[2], alb[3];
    float cw[3];  /* clip weights relative to the source triangle */
    uint32_t src[3];
} rvert;

/* RasterTriangle, RasterTriangle.h:11-24. */
typedef struct
{
    int v0x, v0y, v1x, v1y, v2x, v2y;
    int B0, C0, B1, C1, B2, C2;
    float invDet;
    uint32_t vid[3];
    uint32_t texId;
    unsigned char rej[3], acc[3];
} rtri;

typedef struct
{
    uint32_t tri;
    unsigned char acc[3], trivial, big;
} triref;

typedef struct
{
    const edxr_oracle_params* P;
    const edxr_oracle_mesh* M;
    float mvp[16];
    vec4f* proj;       /* per input vertex */
    rvert* rv; long long nrv, caprv;
    rtri* rt; long long nrt, caprt;
    int tdx, tdy;      /* 32x32 tile grid */
    long long* refStart; /* per tile */
    triref* refs;
    /* padded per-pixel state, (tdx*32) x (tdy*32), one plane per sample */
    int pw, ph;
    int S;             /* samples per pixel */
    size_t npad;       /* pixels of one plane */
    float* depth;
    int* win;          /* raster triangle index or -1 */
    float* l0; float* l1;
    long long* tileFrags;
    double eye[3];
    struct otex* tex; /* texture slots with their mip chains */
} frame;

static int push_rv(frame* f, const rvert* v)
{
    if (f->nrv == f->caprv)
    {
        long long nc = f->caprv ? f->caprv * 2 : 1024;
        rvert* n = (rvert*)realloc(f->rv, (size_t)nc * sizeof(rvert));
        if (!n) return -1;
        f->rv = n; f->caprv = nc;
    }
    f->rv[f->nrv++] = *v;
    return 0;
}

static int push_rt(frame* f, const rtri* t)
{
    if (f->nrt == f->caprt)
    {
        long long nc = f->caprt ? f->caprt * 2 : 1024;
        rtri* n = (rtri*)realloc(f->rt, (size_t)nc * sizeof(rtri));
        if (!n) return -1;
        f->rt = n; f->caprt = nc;
    }
    f->rt[f->nrt++] = *t;
    return 0;
}

static void corner_pair(int B, int C, unsigned char* rej, unsigned char* acc)
{
    /* RasterTriangle.h:66-150: slope = B / float(C), then the sign of C. */
    const float slope = (float)B / (float)C;
    if (slope >= 0.0f)
    {
        if ((float)C >= 0.0f) { *rej = 3; *acc = 0; }
        else { *rej = 0; *acc = 3; }
    }
    else
    {
        if ((float)C >= 0.0f) { *rej = 2; *acc = 1; }
        else { *rej = 1; *acc = 2; }
    }
}

/* RasterTriangle::Setup, RasterTriangle.h:27-153, applied to the projected
 * (not yet post-passed) positions of three raster vertices. */
static int tri_setup(frame* f, uint32_t a, uint32_t b, uint32_t c, uint32_t texId, rtri* t)
{
    const uint32_t ids[3] = { a, b, c };
    int vx[3], vy[3];
    for (int k = 0; k < 3; k++)
    {
        const vec4f p = f->rv[ids[k]].clip;
        const float invW = 1.0f / p.w;
        float r[3];
        xform3_point(f->P->raster, p.x * invW, p.y * invW, p.z * invW, r);
        vx[k] = snap16(r[0]);
        vy[k] = snap16(r[1]);
    }
    t->v0x = vx[0]; t->v0y = vy[0];
    t->v1x = vx[1]; t->v1y = vy[1];
    t->v2x = vx[2]; t->v2y = vy[2];
    t->B0 = wsub(vy[0], vy[1]); t->C0 = wsub(vx[1], vx[0]);
    t->B1 = wsub(vy[1], vy[2]); t->C1 = wsub(vx[2], vx[1]);
    t->B2 = wsub(vy[2], vy[0]); t->C2 = wsub(vx[0], vx[2]);
    const int det = wsub(wmul(t->C2, t->B1), wmul(t->C1, t->B2));
    if (det <= 0)
        return 0;
    t->invDet = 1.0f / (float)det;
    t->vid[0] = a; t->vid[1] = b; t->vid[2] = c;
    t->texId = texId;
    corner_pair(t->B0, t->C0, &t->rej[0], &t->acc[0]);
    corner_pair(t->B1, t->C1, &t->rej[1], &t->acc[1]);
    corner_pair(t->B2, t->C2, &t->rej[2], &t->acc[2]);
    return 1;
}

static void load3(const float* base, int stride, long long i, float out[3], float dflt)
{
    if (!base) { out[0] = out[1] = out[2] = dflt; return; }
    const float* p = base + (size_t)i * stride;
    out[0] = p[0]; out[1] = p[1]; out[2] = p[2];
}

/* Clipper::Clip, Clipper.h:71-189, for all triangles in submission order
 * (the per-core chunks of the reference are contiguous, so concatenating
 * them is submission order), followed by the post-pass of
 * Renderer.cpp:139-147. */
static int stage_clip(frame* f)
{
    const edxr_oracle_mesh* M = f->M;
    for (long long i = 0; i < M->nt; i++)
    {
        const uint32_t* ix = M->indices + 3 * (size_t)i;
        const uint32_t base = (uint32_t)f->nrv;
        for (int k = 0; k < 3; k++)
        {
            rvert v;
            memset(&v, 0, sizeof(v));
            v.clip = f->proj[ix[k]];
            load3(M->positions, M->position_stride, ix[k], v.pos, 0.0f);
            load3(M->normals, M->normal_stride, ix[k], v.nrm, 0.0f);
            load3(M->albedo, M->albedo_stride, ix[k], v.alb, 1.0f);
            if (M->uvs)
            {
                v.uv[0] = M->uvs[(size_t)ix[k] * M->uv_stride];
                v.uv[1] = M->uvs[(size_t)ix[k] * M->uv_stride + 1];
            }
            v.cw[k] = 1.0f;
            v.src[0] = ix[0]; v.src[1] = ix[1]; v.src[2] = ix[2];
            if (push_rv(f, &v)) return -1;
        }
        const vec4f v0 = f->proj[ix[0]], v1 = f->proj[ix[1]], v2 = f->proj[ix[2]];
        const unsigned c0 = clip_code(v0), c1 = clip_code(v1), c2 = clip_code(v2);
        rtri t;
        if (c0 | c1 | c2)
        {
            if (!(c0 & c1 & c2))
            {
                polygon poly;
                poly.n = 3;
                const vec4f vs[3] = { v0, v1, v2 };
                for (int k = 0; k < 3; k++)
                {
                    poly.v[k].pos = vs[k];
                    poly.v[k].w[0] = poly.v[k].w[1] = poly.v[k].w[2] = 0.0f;
                    poly.v[k].w[k] = 1.0f;
                }
                clip_polygon(&poly, (c0 ^ c1) | (c1 ^ c2) | (c2 ^ c0));
                uint32_t ids[MAX_POLY];
                for (int j = 0; j < poly.n; j++)
                {
                    const float* w = poly.v[j].w;
                    if (w[0] == 1.0f) ids[j] = base;
                    else if (w[1] == 1.0f) ids[j] = base + 1;
                    else if (w[2] == 1.0f) ids[j] = base + 2;
                    else
                    {
                        /* Clipper.h:138-151: weight.x*a0 + weight.y*a1 + weight.z*a2 */
                        const rvert* a = &f->rv[base];
                        const rvert* b = &f->rv[base + 1];
                        const rvert* c = &f->rv[base + 2];
                        rvert v;
                        memset(&v, 0, sizeof(v));
                        v.clip = poly.v[j].pos;
                        for (int q = 0; q < 3; q++)
                        {
                            v.pos[q] = w[0] * a->pos[q] + w[1] * b->pos[q] + w[2] * c->pos[q];
                            v.nrm[q] = w[0] * a->nrm[q] + w[1] * b->nrm[q] + w[2] * c->nrm[q];
                            v.alb[q] = w[0] * a->alb[q] + w[1] * b->alb[q] + w[2] * c->alb[q];
                            v.cw[q] = w[q];
                        }
                        for (int q = 0; q < 2; q++)
                            v.uv[q] = w[0] * a->uv[q] + w[1] * b->uv[q] + w[2] * c->uv[q];
                        v.src[0] = ix[0]; v.src[1] = ix[1]; v.src[2] = ix[2];
                        ids[j] = (uint32_t)f->nrv;
                        if (push_rv(f, &v)) return -1;
                    }
                }
                /* Fan triangulation, Clipper.h:156-170. */
                for (int k = 2; k < poly.n; k++)
                    if (tri_setup(f, ids[0], ids[k - 1], ids[k], (uint32_t)i, &t))
                        if (push_rt(f, &t)) return -1;
            }
            continue;
        }
        if (tri_setup(f, base, base + 1, base + 2, (uint32_t)i, &t))
            if (push_rt(f, &t)) return -1;
    }
    /* Post-pass, Renderer.cpp:139-147. */
    for (long long i = 0; i < f->nrv; i++)
    {
        rvert* v = &f->rv[i];
        v->invW = 1.0f / v->clip.w;
        v->clip.z = v->clip.z * v->invW;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Binning, Renderer.cpp:161-229                                              */

/* TopLeftEdge (scalar), RasterTriangle.h:155-158. */
static inline int tl_scalar(int ax, int ay, int bx, int by)
{
    return ((by > ay) || (ay == by && ax > bx)) ? 0 : -1;
}
/* TopLeftEdge (SSE), RasterTriangle.h:296-299, true lanes are -1. */
static inline int tl_sse(int ax, int ay, int bx, int by)
{
    return ((by > ay) || (ay == by && ax > bx)) ? -1 : 0;
}

/* EdgeFunc0..2 (scalar), RasterTriangle.h:160-171. */
static inline int edge_scalar(const rtri* t, int k, int px, int py)
{
    switch (k)
    {
    case 0: return wadd(wadd(wmul(t->B0, wsub(px, t->v0x)), wmul(t->C0, wsub(py, t->v0y))), tl_scalar(t->v0x, t->v0y, t->v1x, t->v1y));
    case 1: return wadd(wadd(wmul(t->B1, wsub(px, t->v1x)), wmul(t->C1, wsub(py, t->v1y))), tl_scalar(t->v1x, t->v1y, t->v2x, t->v2y));
    default: return wadd(wadd(wmul(t->B2, wsub(px, t->v2x)), wmul(t->C2, wsub(py, t->v2y))), tl_scalar(t->v2x, t->v2y, t->v0x, t->v0y));
    }
}

static void bin_tile_range(const frame* f, const rtri* t, int* minX, int* maxX, int* minY, int* maxY)
{
    const int shift = TILE_LOG2 + 4;
    *minX = imax(0, imin(t->v0x, imin(t->v1x, t->v2x)) >> shift);
    *maxX = imin(f->tdx - 1, imax(t->v0x, imax(t->v1x, t->v2x)) >> shift);
    *minY = imax(0, imin(t->v0y, imin(t->v1y, t->v2y)) >> shift);
    *maxY = imin(f->tdy - 1, imax(t->v0y, imax(t->v1y, t->v2y)) >> shift);
}

/* Returns 1 and fills r when triangle t is binned to tile (x, y). */
static int bin_test(const rtri* t, int i, int x, int y, int big, triref* r)
{
    const int shift = TILE_LOG2 + 4;
    r->tri = (uint32_t)i;
    r->big = (unsigned char)big;
    if (!big)
    {
        r->acc[0] = r->acc[1] = r->acc[2] = 0;
        r->trivial = 0;
        return 1;
    }
    for (int k = 0; k < 3; k++)
    {
        const int cx = (x + (t->rej[k] % 2)) << shift;
        const int cy = (y + (t->rej[k] / 2)) << shift;
        if (edge_scalar(t, k, cx, cy) < 0)
            return 0;
    }
    for (int k = 0; k < 3; k++)
    {
        const int cx = (x + (t->acc[k] % 2)) << shift;
        const int cy = (y + (t->acc[k] / 2)) << shift;
        r->acc[k] = edge_scalar(t, k, cx, cy) >= 0;
    }
    r->trivial = r->acc[0] && r->acc[1] && r->acc[2];
    return 1;
}

static int stage_bin(frame* f)
{
    const long long ntiles = (long long)f->tdx * f->tdy;
    long long* cnt = (long long*)calloc((size_t)ntiles + 1, sizeof(long long));
    if (!cnt) return -1;
    for (int pass = 0; pass < 2; pass++)
    {
        for (long long i = 0; i < f->nrt; i++)
        {
            const rtri* t = &f->rt[i];
            int minX, maxX, minY, maxY;
            bin_tile_range(f, t, &minX, &maxX, &minY, &maxY);
            const int big = !(maxX - minX < 2 && maxY - minY < 2);
            for (int y = minY; y <= maxY; y++)
                for (int x = minX; x <= maxX; x++)
                {
                    triref r;
                    if (!bin_test(t, (int)i, x, y, big, &r)) continue;
                    const long long tile = (long long)y * f->tdx + x;
                    if (pass == 0) cnt[tile]++;
                    else f->refs[cnt[tile]++] = r;
                }
        }
        if (pass == 0)
        {
            long long s = 0;
            for (long long k = 0; k < ntiles; k++)
            {
                const long long c = cnt[k];
                f->refStart[k] = s;
                cnt[k] = s;
                s += c;
            }
            f->refStart[ntiles] = s;
            f->refs = (triref*)malloc((size_t)(s ? s : 1) * sizeof(triref));
            if (!f->refs) { free(cnt); return -1; }
        }
    }
    free(cnt);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Rasterization, Rasterizer.h                                                */

/* FrameBuffer::ZTestQuad, FrameBuffer.cpp:54-68 (depth func LEQUAL; LESS is
 * the one-operator variant).  Updates the covered lanes that pass and
 * records the winner; returns the pass mask before the coverage mask. */
static void quad_fragment(frame* f, const rtri* t, int ti, int x, int y, const int covered[4])
{
    static const int offx[4] = { 8, 24, 8, 24 }, offy[4] = { 8, 8, 24, 24 };
    const rvert* v0 = &f->rv[t->vid[0]];
    const rvert* v1 = &f->rv[t->vid[1]];
    const rvert* v2 = &f->rv[t->vid[2]];
    int anyVisible = 0;
    for (int lane = 0; lane < 4; lane++)
    {
        const int cx = (x << 4) + offx[lane], cy = (y << 4) + offy[lane];
        /* TriangleSSE::CalcBarycentricCoord, RasterTriangle.h:333-337 */
        const int e1 = wadd(wmul(t->B1, wsub(cx, t->v2x)), wmul(t->C1, wsub(cy, t->v2y)));
        const int e2 = wadd(wmul(t->B2, wsub(cx, t->v2x)), wmul(t->C2, wsub(cy, t->v2y)));
        const float l0 = (float)e1 * t->invDet;
        const float l1 = (float)e2 * t->invDet;
        /* TriangleSSE::GetDepth, RasterTriangle.h:324-331 */
        const float l2 = (1.0f - l0) - l1;
        const float d = (l0 * v0->clip.z + l1 * v1->clip.z) + l2 * v2->clip.z;
        const int px = x + (lane & 1), py = y + (lane >> 1);
        const size_t p = (size_t)py * f->pw + px;
        const float cur = f->depth[p];
        const int pass = (f->P->depth_func == EDXR_ORACLE_DEPTH_LESS) ? (d < cur) : (d <= cur);
        if (pass && covered[lane])
        {
            f->depth[p] = d;
            f->win[p] = ti;
            f->l0[p] = l0;
            f->l1[p] = l1;
            anyVisible = 1;
        }
    }
    if (anyVisible)
        f->tileFrags[(y >> TILE_LOG2) * f->tdx + (x >> TILE_LOG2)]++;
}

/* FrameBuffer::MultiSampleOffsets (FrameBuffer.cpp:107-191): the table of
 * 1/16-pixel sample offsets, per sample-count log2, as the reference lists
 * it.  The rasterizer reads sample s as `const Vector2i& sampleOffset =
 * MultiSampleOffsets[level][2 * s]` (Rasterizer.h:247, 382): an int bound to
 * a Vector2i reference goes through Vector2i's scalar constructor, so the
 * sample sits at (t[2s], t[2s]) from the pixel centre.  sample_offset() is
 * that value. */
static const int kSampleOffsets[6][64] = {
    { 0, 0 },
    { 4, 4, -4, -4 },
    { -2, -6, 6, -2, -6, 2, 2, 6 },
    { 1, -3, -1, 3, 5, 1, -3, -5, -5, 5, -7, -1, 3, 7, 7, -7 },
    { 1, 1, -1, -3, -3, 2, 4, -1, -5, -2, 2, 5, 5, 3, 3, -5,
      -2, 6, 0, -7, -4, -6, -6, 4, -8, 0, 7, -4, 6, 7, -7, -8 },
    { 1, 1, -1, -3, -3, 2, 4, -1, -5, -2, 2, 5, 5, 3, 3, -5,
      -2, 6, 0, -7, -4, -6, -6, 4, -8, 0, 7, -4, 6, 7, -7, -8,
      1, 3, -3, -3, -3, 0, 6, -2, -7, -1, 3, 4, 7, 3, 3, -6,
      -2, 7, 0, -4, -2, -5, -7, 6, -8, 3, 4, -1, 2, 7, 4, -8 }
};

static inline int sample_offset(int level, int s) { return kSampleOffsets[level][2 * s]; }

/* Depth test of one sample at 1/16-pixel position (sx, sy) (ZTestQuad with a
 * sample id, FrameBuffer.cpp:54-68; the depth from the sample's barycentrics,
 * RasterTriangle.h:324-337).  Returns whether the sample passed. */
static int sample_test(frame* f, const rtri* t, int ti, int px, int py, int s, int sx, int sy)
{
    const rvert* v0 = &f->rv[t->vid[0]];
    const rvert* v1 = &f->rv[t->vid[1]];
    const rvert* v2 = &f->rv[t->vid[2]];
    const int e1 = wadd(wmul(t->B1, wsub(sx, t->v2x)), wmul(t->C1, wsub(sy, t->v2y)));
    const int e2 = wadd(wmul(t->B2, wsub(sx, t->v2x)), wmul(t->C2, wsub(sy, t->v2y)));
    const float l0 = (float)e1 * t->invDet;
    const float l1 = (float)e2 * t->invDet;
    const float l2 = (1.0f - l0) - l1;
    const float d = (l0 * v0->clip.z + l1 * v1->clip.z) + l2 * v2->clip.z;
    const size_t p = (size_t)s * f->npad + (size_t)py * f->pw + px;
    const float cur = f->depth[p];
    const int pass = (f->P->depth_func == EDXR_ORACLE_DEPTH_LESS) ? (d < cur) : (d <= cur);
    if (pass)
    {
        f->depth[p] = d;
        f->win[p] = ti;
    }
    return pass;
}

/* Rasterizer::FineRasterize_MultiSample, Rasterizer.h:202-300: per sample the
 * biased pixel-centre edge values plus the sample offset, then the sample's
 * depth test. */
static void fine_raster_ms(frame* f, const rtri* t, int ti, int minX, int minY, int maxX, int maxY)
{
    static const int offx[4] = { 8, 24, 8, 24 }, offy[4] = { 8, 8, 24, 24 };
    const int level = f->P->msaa_log2;
    const int b0 = tl_sse(t->v0x, t->v0y, t->v1x, t->v1y);
    const int b1 = tl_sse(t->v1x, t->v1y, t->v2x, t->v2y);
    const int b2 = tl_sse(t->v2x, t->v2y, t->v0x, t->v0y);
    for (int y = minY; y <= maxY; y += 2)
        for (int x = minX; x <= maxX; x += 2)
        {
            int any = 0;
            for (int lane = 0; lane < 4; lane++)
            {
                const int cx = (x << 4) + offx[lane], cy = (y << 4) + offy[lane];
                const int e0 = wadd(wadd(wmul(t->B0, wsub(cx, t->v0x)), wmul(t->C0, wsub(cy, t->v0y))), b0);
                const int e1 = wadd(wadd(wmul(t->B1, wsub(cx, t->v1x)), wmul(t->C1, wsub(cy, t->v1y))), b1);
                const int e2 = wadd(wadd(wmul(t->B2, wsub(cx, t->v2x)), wmul(t->C2, wsub(cy, t->v2y))), b2);
                for (int s = 0; s < f->S; s++)
                {
                    const int ox = sample_offset(level, s), oy = ox;
                    const int s0 = wadd(wadd(e0, wmul(ox, t->B0)), wmul(oy, t->C0));
                    const int s1 = wadd(wadd(e1, wmul(ox, t->B1)), wmul(oy, t->C1));
                    const int s2 = wadd(wadd(e2, wmul(ox, t->B2)), wmul(oy, t->C2));
                    if ((s0 | s1 | s2) >= 0)
                        any |= sample_test(f, t, ti, x + (lane & 1), y + (lane >> 1), s, cx + ox, cy + oy);
                }
            }
            if (any)
                f->tileFrags[(y >> TILE_LOG2) * f->tdx + (x >> TILE_LOG2)]++;
        }
}

/* Rasterizer::TrivialAcceptTriangle_MultiSample, Rasterizer.h:355-415. */
static void trivial_accept_ms(frame* f, const rtri* t, int ti, int minX, int minY, int maxX, int maxY)
{
    static const int offx[4] = { 8, 24, 8, 24 }, offy[4] = { 8, 8, 24, 24 };
    const int level = f->P->msaa_log2;
    for (int y = minY; y <= maxY; y += 2)
        for (int x = minX; x <= maxX; x += 2)
        {
            int any = 0;
            for (int lane = 0; lane < 4; lane++)
            {
                const int cx = (x << 4) + offx[lane], cy = (y << 4) + offy[lane];
                for (int s = 0; s < f->S; s++)
                {
                    const int o = sample_offset(level, s);
                    any |= sample_test(f, t, ti, x + (lane & 1), y + (lane >> 1), s, cx + o, cy + o);
                }
            }
            if (any)
                f->tileFrags[(y >> TILE_LOG2) * f->tdx + (x >> TILE_LOG2)]++;
        }
}

/* Rasterizer::FineRasterize_SingleSample, Rasterizer.h:126-200. */
static void fine_raster(frame* f, const rtri* t, int ti, int bminx, int bminy, int bmaxx, int bmaxy)
{
    int minX = imax(bminx, imin(t->v0x, imin(t->v1x, t->v2x)) >> 4);
    int maxX = imin(bmaxx - 1, imax(t->v0x, imax(t->v1x, t->v2x)) >> 4);
    int minY = imax(bminy, imin(t->v0y, imin(t->v1y, t->v2y)) >> 4);
    int maxY = imin(bmaxy - 1, imax(t->v0y, imax(t->v1y, t->v2y)) >> 4);
    minX -= minX % 2;
    minY -= minY % 2;
    if (maxX < minX || maxY < minY)
        return;
    if (f->S > 1)
    {
        fine_raster_ms(f, t, ti, minX, minY, maxX, maxY);
        return;
    }
    static const int offx[4] = { 8, 24, 8, 24 }, offy[4] = { 8, 8, 24, 24 };
    const int b0 = tl_sse(t->v0x, t->v0y, t->v1x, t->v1y);
    const int b1 = tl_sse(t->v1x, t->v1y, t->v2x, t->v2y);
    const int b2 = tl_sse(t->v2x, t->v2y, t->v0x, t->v0y);
    for (int y = minY; y <= maxY; y += 2)
        for (int x = minX; x <= maxX; x += 2)
        {
            int covered[4], any = 0;
            for (int lane = 0; lane < 4; lane++)
            {
                const int cx = (x << 4) + offx[lane], cy = (y << 4) + offy[lane];
                /* Incremental stepping in the reference equals direct
                 * evaluation modulo 2^32. */
                const int e0 = wadd(wadd(wmul(t->B0, wsub(cx, t->v0x)), wmul(t->C0, wsub(cy, t->v0y))), b0);
                const int e1 = wadd(wadd(wmul(t->B1, wsub(cx, t->v1x)), wmul(t->C1, wsub(cy, t->v1y))), b1);
                const int e2 = wadd(wadd(wmul(t->B2, wsub(cx, t->v2x)), wmul(t->C2, wsub(cy, t->v2y))), b2);
                covered[lane] = (e0 | e1 | e2) >= 0;
                any |= covered[lane];
            }
            if (any)
                quad_fragment(f, t, ti, x, y, covered);
        }
}

/* Rasterizer::TrivialAcceptTriangle_SingleSample, Rasterizer.h:310-353. */
static void trivial_accept(frame* f, const rtri* t, int ti, int bminx, int bminy, int bmaxx, int bmaxy)
{
    int minX = bminx, maxX = bmaxx - 1, minY = bminy, maxY = bmaxy - 1;
    minX -= minX % 2;
    minY -= minY % 2;
    if (f->S > 1)
    {
        trivial_accept_ms(f, t, ti, minX, minY, maxX, maxY);
        return;
    }
    static const int all[4] = { 1, 1, 1, 1 };
    for (int y = minY; y <= maxY; y += 2)
        for (int x = minX; x <= maxX; x += 2)
            quad_fragment(f, t, ti, x, y, all);
}

/* GenStepVectors, RasterTriangle.h:192-255: per quadrant offsets of the
 * corner's edge value, each lane = stepSize * (lane value). */
static void step_vec(int corner, int B, int C, int stepSize, int out[4])
{
    int v[4];
    switch (corner)
    {
    case 0: v[0] = 0; v[1] = B; v[2] = C; v[3] = wadd(B, C); break;
    case 1: v[0] = wsub(0, B); v[1] = 0; v[2] = wsub(C, B); v[3] = C; break;
    case 2: v[0] = wsub(0, C); v[1] = wsub(B, C); v[2] = 0; v[3] = B; break;
    default: v[0] = wsub(wsub(0, B), C); v[1] = wsub(0, C); v[2] = wsub(0, B); v[3] = 0; break;
    }
    for (int i = 0; i < 4; i++)
        out[i] = wmul(stepSize, v[i]);
}

/* Rasterizer::CoarseRasterize, Rasterizer.h:32-111 (single sample). */
static void coarse_raster(frame* f, const triref* r, const rtri* t, int ti, int blockSize,
                          int bminx, int bminy, int bmaxx, int bmaxy)
{
    const int baseX = bminx << 4, baseY = bminy << 4;
    const int span = (blockSize << 4) - 1;
    const int Bs[3] = { t->B0, t->B1, t->B2 }, Cs[3] = { t->C0, t->C1, t->C2 };
    int rejE[3][4], accE[3][4];
    for (int k = 0; k < 3; k++)
    {
        int rs[4], as[4];
        step_vec(t->rej[k], Bs[k], Cs[k], blockSize << 3, rs);
        step_vec(t->acc[k], Bs[k], Cs[k], blockSize << 3, as);
        const int re = edge_scalar(t, k, baseX + (t->rej[k] % 2) * span, baseY + (t->rej[k] >> 1) * span);
        for (int q = 0; q < 4; q++)
            rejE[k][q] = wadd(re, rs[q]);
        if (!r->acc[k])
        {
            const int ae = edge_scalar(t, k, baseX + (t->acc[k] % 2) * span, baseY + (t->acc[k] >> 1) * span);
            for (int q = 0; q < 4; q++)
                accE[k][q] = wadd(ae, as[q]);
        }
        else
            for (int q = 0; q < 4; q++)
                accE[k][q] = INT_MAX; /* IntSSE(EDX_INFINITY) */
    }
    const int half = blockSize >> 1;
    for (int q = 0; q < 4; q++)
    {
        if (rejE[0][q] < 0 || rejE[1][q] < 0 || rejE[2][q] < 0)
            continue;
        const int minX = !(q % 2) ? bminx : bminx + half;
        const int maxX = !(q % 2) ? bminx + half : bmaxx;
        const int minY = !(q >> 1) ? bminy : bminy + half;
        const int maxY = !(q >> 1) ? bminy + half : bmaxy;
        if (accE[0][q] >= 0 && accE[1][q] >= 0 && accE[2][q] >= 0)
            trivial_accept(f, t, ti, minX, minY, maxX, maxY);
        else
            fine_raster(f, t, ti, minX, minY, maxX, maxY);
    }
}

/* Renderer::RasterizeTile, Renderer.cpp:248-270. */
static void raster_tile(frame* f, long long tile)
{
    const int tx = (int)(tile % f->tdx), ty = (int)(tile / f->tdx);
    const int minX = tx * TILE_SIZE, minY = ty * TILE_SIZE;
    const int maxX = imin(minX + TILE_SIZE, f->P->width), maxY = imin(minY + TILE_SIZE, f->P->height);
    for (long long j = f->refStart[tile]; j < f->refStart[tile + 1]; j++)
    {
        const triref* r = &f->refs[j];
        const rtri* t = &f->rt[r->tri];
        if (r->trivial)
            trivial_accept(f, t, (int)r->tri, minX, minY, maxX, maxY);
        else if (f->P->hierarchical && r->big)
            coarse_raster(f, r, t, (int)r->tri, TILE_SIZE, minX, minY, maxX, maxY);
        else
            fine_raster(f, t, (int)r->tri, minX, minY, maxX, maxY);
    }
}

/* ------------------------------------------------------------------------ */
/* Shading (FP64)                                                             */

static double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void normalize3(double v[3])
{
    const double l = sqrt(dot3(v, v));
    v[0] /= l; v[1] /= l; v[2] /= l;
}

void edxr_oracle_shade(const edxr_oracle_params* P, const double b[3],
                       const double pos[3][3], const double nrm[3][3],
                       const double alb[3][3], const double eye[3], double rgb[3])
{
    double Pp[3], N[3], A[3];
    for (int q = 0; q < 3; q++)
    {
        Pp[q] = b[0] * pos[0][q] + b[1] * pos[1][q] + b[2] * pos[2][q];
        N[q] = b[0] * nrm[0][q] + b[1] * nrm[1][q] + b[2] * nrm[2][q];
        A[q] = b[0] * alb[0][q] + b[1] * alb[1][q] + b[2] * alb[2][q];
    }
    normalize3(N);
    double L[3] = { P->light[0], P->light[1], P->light[2] };
    normalize3(L);
    double nl = dot3(L, N);
    if (nl < 0.0) nl = 0.0;
    /* (max(N.L, 0) + 0.2) * 3 / pi, Shader.h:260-264 */
    const double diffuse = (nl + 0.2) * 3.0 / 3.14159265358979323846;
    double spec = 0.0;
    if (P->shader == EDXR_ORACLE_PS_BLINN_PHONG || P->shader == EDXR_ORACLE_PS_BLINN_PHONG_REFERENCE)
    {
        /* Shader.h:266-278 */
        double E[3] = { eye[0] - Pp[0], eye[1] - Pp[1], eye[2] - Pp[2] };
        normalize3(E);
        double H[3] = { L[0] + E[0], L[1] + E[1], L[2] + E[2] };
        normalize3(H);
        double nh = dot3(N, H);
        if (P->shader == EDXR_ORACLE_PS_BLINN_PHONG && nh < 0.0) nh = 0.0;
        spec = (double)P->ks * pow(nh, (double)P->shininess);
    }
    switch (P->shader)
    {
    case EDXR_ORACLE_PS_BLINN_PHONG:
        for (int q = 0; q < 3; q++) rgb[q] = A[q] * diffuse + spec;
        break;
    case EDXR_ORACLE_PS_BLINN_PHONG_REFERENCE:
        for (int q = 0; q < 3; q++) rgb[q] = diffuse + spec;
        break;
    case EDXR_ORACLE_PS_LAMBERTIAN_ALBEDO:
    case EDXR_ORACLE_PS_LAMBERTIAN_TEXTURED:
        for (int q = 0; q < 3; q++) rgb[q] = A[q] * diffuse;
        break;
    default:
        for (int q = 0; q < 3; q++) rgb[q] = diffuse;
        break;
    }
}

/* ------------------------------------------------------------------------ */
/* Texture sampling of the textured Lambertian shader (Shader.h:226-239).
 * EDXUtil's sampler is absent; this is the build's contract, restated in
 * FP32 with the kernels' operations: coordinates repeat; nearest and bilinear
 * sample level 0; trilinear blends the bilinear samples of the two levels
 * around lod = 0.5 log2(max |d|^2) (differentials in texels); anisotropic Nx
 * averages n = min(N, ceil(major / minor)) trilinear probes along the longer
 * differential at the lod of major / n.  Mip level l+1 texel = mean of the
 * 2x2 texels of level l (indices clamped), summed in order then times 0.25. */
typedef struct otex
{
    int w, h, levels;
    float* texels; /* RGBA, all levels one after the other */
} otex;

typedef struct
{
    const float* t;
    int w, h;
} olevel;

static olevel tex_level(const otex* x, int level)
{
    size_t off = 0;
    int w = x->w, h = x->h;
    for (int l = 0; l < level; l++)
    {
        off += (size_t)w * h;
        w = w > 1 ? w >> 1 : 1;
        h = h > 1 ? h >> 1 : 1;
    }
    olevel L = { x->texels + 4 * off, w, h };
    return L;
}

static int build_texture(const edxr_oracle_texture* in, otex* out)
{
    size_t total = 0;
    int w = in->width, h = in->height, levels = 1;
    total += (size_t)w * h;
    while (w > 1 || h > 1)
    {
        w = w > 1 ? w >> 1 : 1;
        h = h > 1 ? h >> 1 : 1;
        total += (size_t)w * h;
        levels++;
    }
    out->w = in->width;
    out->h = in->height;
    out->levels = levels;
    out->texels = (float*)malloc(total * 4 * sizeof(float));
    if (!out->texels) return -1;
    const size_t n0 = (size_t)in->width * in->height;
    for (size_t k = 0; k < 4 * n0; k++)
        out->texels[k] = in->format == 0 ? ((const unsigned char*)in->texels)[k] / 255.0f
                                         : ((const float*)in->texels)[k];
    for (int l = 1; l < levels; l++)
    {
        const olevel a = tex_level(out, l - 1), b = tex_level(out, l);
        float* dst = (float*)b.t;
        for (int y = 0; y < b.h; y++)
            for (int x = 0; x < b.w; x++)
            {
                const int x0 = imin(2 * x, a.w - 1), x1 = imin(2 * x + 1, a.w - 1);
                const int y0 = imin(2 * y, a.h - 1), y1 = imin(2 * y + 1, a.h - 1);
                for (int c = 0; c < 4; c++)
                {
                    const float s = ((a.t[4 * ((size_t)y0 * a.w + x0) + c] + a.t[4 * ((size_t)y0 * a.w + x1) + c]) +
                                     a.t[4 * ((size_t)y1 * a.w + x0) + c]) + a.t[4 * ((size_t)y1 * a.w + x1) + c];
                    dst[4 * ((size_t)y * b.w + x) + c] = s * 0.25f;
                }
            }
    }
    return 0;
}

static float wrap01(float u) { return u - floorf(u); }
static float lerpf(float a, float b, float t) { return fmaf(t, b - a, a); }

static void tex_fetch(const olevel* L, int x, int y, float c[4])
{
    x %= L->w;
    if (x < 0) x += L->w;
    y %= L->h;
    if (y < 0) y += L->h;
    const float* p = L->t + 4 * ((size_t)y * L->w + x);
    for (int k = 0; k < 4; k++) c[k] = p[k];
}

static void tex_bilinear(const olevel* L, float u, float v, float c[4])
{
    const float fx = wrap01(u) * (float)L->w - 0.5f, fy = wrap01(v) * (float)L->h - 0.5f;
    const float x0 = floorf(fx), y0 = floorf(fy);
    const float tx = fx - x0, ty = fy - y0;
    const int ix = (int)x0, iy = (int)y0;
    float a[4], b[4], p[4], q[4];
    tex_fetch(L, ix, iy, a);
    tex_fetch(L, ix + 1, iy, b);
    tex_fetch(L, ix, iy + 1, p);
    tex_fetch(L, ix + 1, iy + 1, q);
    for (int k = 0; k < 4; k++)
        c[k] = lerpf(lerpf(a[k], b[k], tx), lerpf(p[k], q[k], tx), ty);
}

static void tex_trilinear(const otex* x, float u, float v, float lod, float c[4])
{
    lod = fminf(fmaxf(lod, 0.0f), (float)(x->levels - 1));
    const int l0 = (int)floorf(lod);
    const float t = lod - (float)l0;
    olevel L0 = tex_level(x, l0);
    tex_bilinear(&L0, u, v, c);
    if (t == 0.0f)
        return;
    olevel L1 = tex_level(x, imin(l0 + 1, x->levels - 1));
    float d[4];
    tex_bilinear(&L1, u, v, d);
    for (int k = 0; k < 4; k++) c[k] = lerpf(c[k], d[k], t);
}

static void sample_texture(const otex* x, int filter, float u, float v, const float d0[2], const float d1[2],
                           float c[4])
{
    if (filter == 0)
    {
        olevel L = tex_level(x, 0);
        const int ix = imin((int)floorf(wrap01(u) * (float)L.w), L.w - 1);
        const int iy = imin((int)floorf(wrap01(v) * (float)L.h), L.h - 1);
        tex_fetch(&L, ix, iy, c);
        return;
    }
    if (filter == 1)
    {
        olevel L = tex_level(x, 0);
        tex_bilinear(&L, u, v, c);
        return;
    }
    const float ax = d0[0] * (float)x->w, ay = d0[1] * (float)x->h;
    const float bx = d1[0] * (float)x->w, by = d1[1] * (float)x->h;
    const float r0 = fmaf(ax, ax, ay * ay), r1 = fmaf(bx, bx, by * by);
    if (filter == 2)
    {
        const float r = fmaxf(r0, r1);
        tex_trilinear(x, u, v, r > 1.0f ? 0.5f * log2f(r) : 0.0f, c);
        return;
    }
    const int N = filter == 3 ? 4 : (filter == 4 ? 8 : 16);
    const float l0 = sqrtf(r0), l1 = sqrtf(r1);
    const float major = fmaxf(l0, l1), minor = fminf(l0, l1);
    const int n = major <= 0.0f ? 1 : (minor <= 0.0f ? N : imin(N, (int)ceilf(major / minor)));
    const float* axis = l0 >= l1 ? d0 : d1;
    const float m = major / (float)n;
    const float lod = m > 1.0f ? log2f(m) : 0.0f;
    float acc[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
    for (int i = 0; i < n; i++)
    {
        const float sft = ((float)i + 0.5f) / (float)n - 0.5f;
        float p[4];
        tex_trilinear(x, fmaf(axis[0], sft, u), fmaf(axis[1], sft, v), lod, p);
        for (int k = 0; k < 4; k++) acc[k] = acc[k] + p[k];
    }
    const float inv = 1.0f / (float)n;
    for (int k = 0; k < 4; k++) c[k] = acc[k] * inv;
}

/* Perspective-correct barycentrics of raster triangle t at the centre of
 * pixel (px, py), in float as the kernels form them (RasterTriangle.h:333-337,
 * Shader.h:150-158). */
static void persp_bary(const frame* f, const rtri* t, int px, int py, float b[3])
{
    const int cx = (px << 4) + 8, cy = (py << 4) + 8;
    const int e1 = wadd(wmul(t->B1, wsub(cx, t->v2x)), wmul(t->C1, wsub(cy, t->v2y)));
    const int e2 = wadd(wmul(t->B2, wsub(cx, t->v2x)), wmul(t->C2, wsub(cy, t->v2y)));
    float b0 = (float)e1 * t->invDet, b1 = (float)e2 * t->invDet;
    float b2 = (1.0f - b0) - b1;
    b0 = b0 * f->rv[t->vid[0]].invW;
    b1 = b1 * f->rv[t->vid[1]].invW;
    b2 = b2 * f->rv[t->vid[2]].invW;
    const float invB = 1.0f / ((b0 + b1) + b2);
    b0 = b0 * invB;
    b1 = b1 * invB;
    b[0] = b0;
    b[1] = b1;
    b[2] = (1.0f - b0) - b1;
}

/* Albedo of the textured shader at pixel (px, py): the texture coordinate
 * there and the differentials of the pixel's 2x2 quad (lane 1 - lane 0,
 * lane 2 - lane 0; Shader.h:226-228). */
static void texture_albedo(const frame* f, int ti, int px, int py, double alb[3])
{
    const rtri* t = &f->rt[ti];
    const edxr_oracle_mesh* M = f->M;
    const uint32_t slot = M->texture_ids ? M->texture_ids[t->texId] : 0u;
    if (slot >= (uint32_t)f->P->num_textures || !M->uvs)
    {
        alb[0] = alb[1] = alb[2] = 1.0;
        return;
    }
    const float* uv[3] = { f->rv[t->vid[0]].uv, f->rv[t->vid[1]].uv, f->rv[t->vid[2]].uv };
    float q[4][2];
    const int qx = px & ~1, qy = py & ~1;
    const int lx[4] = { qx, qx + 1, qx, px }, ly[4] = { qy, qy, qy + 1, py };
    for (int k = 0; k < 4; k++)
    {
        float b[3];
        persp_bary(f, t, lx[k], ly[k], b);
        for (int c = 0; c < 2; c++)
            q[k][c] = fmaf(b[0], uv[0][c], fmaf(b[1], uv[1][c], b[2] * uv[2][c]));
    }
    const float d0[2] = { q[1][0] - q[0][0], q[1][1] - q[0][1] };
    const float d1[2] = { q[2][0] - q[0][0], q[2][1] - q[0][1] };
    float c[4];
    sample_texture(&f->tex[slot], f->P->texture_filter, q[3][0], q[3][1], d0, d1, c);
    alb[0] = c[0];
    alb[1] = c[1];
    alb[2] = c[2];
}

/* Fragment::Interpolate (Shader.h:142-170) in FP64 from the winner's float
 * barycentrics, then the shading model; the textured shader's albedo is the
 * texture sample at pixel (px, py). */
static void shade_pixel(const frame* f, int ti, float l0, float l1, int px, int py, double rgb[3])
{
    const rtri* t = &f->rt[ti];
    const edxr_oracle_mesh* M = f->M;
    double b[3] = { (double)l0, (double)l1, 0.0 };
    b[2] = 1.0 - b[0] - b[1];
    double pos[3][3], nrm[3][3], alb[3][3];
    for (int k = 0; k < 3; k++)
    {
        const rvert* v = &f->rv[t->vid[k]];
        b[k] *= 1.0 / (double)v->clip.w;
        for (int q = 0; q < 3; q++) pos[k][q] = nrm[k][q] = alb[k][q] = 0.0;
        for (int s = 0; s < 3; s++)
        {
            const double w = (double)v->cw[s];
            float sp[3], sn[3], sa[3];
            load3(M->positions, M->position_stride, v->src[s], sp, 0.0f);
            load3(M->normals, M->normal_stride, v->src[s], sn, 0.0f);
            load3(M->albedo, M->albedo_stride, v->src[s], sa, 1.0f);
            for (int q = 0; q < 3; q++)
            {
                pos[k][q] += w * sp[q];
                nrm[k][q] += w * sn[q];
                alb[k][q] += w * sa[q];
            }
        }
    }
    const double s = 1.0 / (b[0] + b[1] + b[2]);
    b[0] *= s;
    b[1] *= s;
    b[2] = 1.0 - b[0] - b[1];
    if (f->P->shader == EDXR_ORACLE_PS_LAMBERTIAN_TEXTURED)
    {
        double a[3];
        texture_albedo(f, ti, px, py, a);
        for (int k = 0; k < 3; k++)
            for (int q = 0; q < 3; q++)
                alb[k][q] = a[q];
    }
    edxr_oracle_shade(f->P, b, pos, nrm, alb, f->eye, rgb);
}

/* Eye position MV^-1 * 0 (Renderer.cpp:289), in double. */
static void eye_position(const float* mv, double eye[3])
{
    double a[4][8];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
        {
            a[i][j] = mv[i * 4 + j];
            a[i][j + 4] = (i == j) ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; c++)
    {
        int piv = c;
        for (int r = c + 1; r < 4; r++)
            if (fabs(a[r][c]) > fabs(a[piv][c])) piv = r;
        if (piv != c)
            for (int j = 0; j < 8; j++) { double tt = a[c][j]; a[c][j] = a[piv][j]; a[piv][j] = tt; }
        const double d = a[c][c];
        for (int j = 0; j < 8; j++) a[c][j] /= d;
        for (int r = 0; r < 4; r++)
        {
            if (r == c) continue;
            const double m = a[r][c];
            for (int j = 0; j < 8; j++) a[r][j] -= m * a[c][j];
        }
    }
    const double w = a[3][7];
    eye[0] = a[0][7] / w;
    eye[1] = a[1][7] / w;
    eye[2] = a[2][7] / w;
}

/* ------------------------------------------------------------------------ */
/* Thread pool over an index range                                            */

typedef struct
{
    frame* f;
    long long next, end;
    int kind; /* 0 raster tiles, 1 shade rows */
    edxr_oracle_out* out;
} job;

/* Color4b::FromFloats / Color4b(Color) of the shim: clamp, scale by 255,
 * round half up, all in float. */
static unsigned char to_byte(float v)
{
    v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
    return (unsigned char)(v * 255.0f + 0.5f);
}

/* One pixel with S > 1 samples: every sample's winner is shaded at the pixel
 * centre (the fragment's barycentrics, Rasterizer.h:279-281), stored as 8-bit
 * colour (Renderer.cpp:295-299, 305-350; a sample no fragment reached keeps
 * the clear value 0), and FrameBuffer::Resolve (FrameBuffer.cpp:70-87)
 * averages the samples in float. */
static void shade_pixel_ms(frame* f, edxr_oracle_out* out, int x, int y)
{
    const int W = f->P->width, H = f->P->height;
    const size_t po = (size_t)y * W + x;
    float acc[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
    for (int s = 0; s < f->S; s++)
    {
        const size_t pp = (size_t)s * f->npad + (size_t)y * f->pw + x;
        const size_t so = (size_t)s * W * H + po;
        const int ti = f->win[pp];
        if (out->id) out->id[so] = ti < 0 ? 0xFFFFFFFFu : f->rt[ti].texId;
        if (out->depth) out->depth[so] = f->depth[pp];
        if (ti < 0 || !out->color)
            continue;
        const rtri* t = &f->rt[ti];
        const int cx = (x << 4) + 8, cy = (y << 4) + 8;
        const int e1 = wadd(wmul(t->B1, wsub(cx, t->v2x)), wmul(t->C1, wsub(cy, t->v2y)));
        const int e2 = wadd(wmul(t->B2, wsub(cx, t->v2x)), wmul(t->C2, wsub(cy, t->v2y)));
        double rgb[3];
        shade_pixel(f, ti, (float)e1 * t->invDet, (float)e2 * t->invDet, x, y, rgb);
        for (int q = 0; q < 3; q++)
            acc[q] += (float)to_byte((float)rgb[q]) / 255.0f;
        acc[3] += 255.0f / 255.0f;
    }
    if (out->color)
    {
        const float inv = 1.0f / (float)f->S;
        for (int q = 0; q < 4; q++)
            out->color[4 * po + q] = (double)(acc[q] * inv);
    }
}

static void shade_row(frame* f, edxr_oracle_out* out, int y)
{
    const int W = f->P->width;
    if (f->S > 1)
    {
        for (int x = 0; x < W; x++)
            shade_pixel_ms(f, out, x, y);
        return;
    }
    for (int x = 0; x < W; x++)
    {
        const size_t pp = (size_t)y * f->pw + x;
        const size_t po = (size_t)y * W + x;
        const int ti = f->win[pp];
        if (out->id) out->id[po] = ti < 0 ? 0xFFFFFFFFu : f->rt[ti].texId;
        if (out->depth) out->depth[po] = f->depth[pp];
        if (out->lambda0) out->lambda0[po] = ti < 0 ? 0.0f : f->l0[pp];
        if (out->lambda1) out->lambda1[po] = ti < 0 ? 0.0f : f->l1[pp];
        if (out->color)
        {
            double* c = out->color + 4 * po;
            if (ti < 0)
                c[0] = c[1] = c[2] = c[3] = 0.0;
            else
            {
                shade_pixel(f, ti, f->l0[pp], f->l1[pp], x, y, c);
                c[3] = 1.0;
            }
        }
    }
}

static void* worker(void* arg)
{
    job* j = (job*)arg;
    for (;;)
    {
        const long long i = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
        if (i >= j->end) break;
        if (j->kind == 0) raster_tile(j->f, i);
        else shade_row(j->f, j->out, (int)i);
    }
    return NULL;
}

static void run_parallel(frame* f, edxr_oracle_out* out, int kind, long long n, int threads)
{
    job j = { f, 0, n, kind, out };
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t th[256];
    int started = 0;
    for (int i = 1; i < threads; i++)
        if (pthread_create(&th[started], NULL, worker, &j) == 0) started++;
    worker(&j);
    for (int i = 0; i < started; i++)
        pthread_join(th[i], NULL);
}

/* ------------------------------------------------------------------------ */

int edxr_oracle_render(const edxr_oracle_params* P, const edxr_oracle_mesh* M, edxr_oracle_out* out)
{
    if (!P || !M || !out || P->width <= 0 || P->height <= 0 || M->nv < 0 || M->nt < 0 ||
        P->msaa_log2 < 0 || P->msaa_log2 > 5)
        return -1;
    if (M->nt > 0 && (!M->indices || !M->positions))
        return -1;
    for (long long i = 0; i < 3LL * M->nt; i++)
        if (M->indices[i] >= (uint32_t)M->nv)
            return -2;

    frame f;
    memset(&f, 0, sizeof(f));
    f.P = P;
    f.M = M;
    int rc = -3;
    if (P->num_textures > 0)
    {
        f.tex = (otex*)calloc((size_t)P->num_textures, sizeof(otex));
        if (!f.tex) goto done;
        for (int i = 0; i < P->num_textures; i++)
            if (build_texture(&P->textures[i], &f.tex[i])) goto done;
    }
    mat_mul(P->proj, P->mv, f.mvp);
    eye_position(P->mv, f.eye);

    /* Vertex stage, Renderer.cpp:120-127 / Shader.h:40-49. */
    f.proj = (vec4f*)malloc((size_t)(M->nv ? M->nv : 1) * sizeof(vec4f));
    if (!f.proj) goto done;
    for (long long i = 0; i < M->nv; i++)
    {
        const float* p = M->positions + (size_t)i * M->position_stride;
        f.proj[i] = xform4(f.mvp, p[0], p[1], p[2]);
    }
    if (stage_clip(&f)) goto done;

    f.tdx = (P->width + TILE_SIZE - 1) >> TILE_LOG2;
    f.tdy = (P->height + TILE_SIZE - 1) >> TILE_LOG2;
    const long long ntiles = (long long)f.tdx * f.tdy;
    f.refStart = (long long*)calloc((size_t)ntiles + 1, sizeof(long long));
    f.tileFrags = (long long*)calloc((size_t)ntiles, sizeof(long long));
    if (!f.refStart || !f.tileFrags) goto done;
    if (stage_bin(&f)) goto done;

    f.pw = f.tdx * TILE_SIZE;
    f.ph = f.tdy * TILE_SIZE;
    f.S = 1 << P->msaa_log2;
    const size_t npad = (size_t)f.pw * f.ph;
    f.npad = npad;
    f.depth = (float*)malloc(npad * f.S * sizeof(float));
    f.win = (int*)malloc(npad * f.S * sizeof(int));
    f.l0 = (float*)malloc(npad * sizeof(float));
    f.l1 = (float*)malloc(npad * sizeof(float));
    if (!f.depth || !f.win || !f.l0 || !f.l1) goto done;
    for (size_t i = 0; i < npad * f.S; i++)
    {
        f.depth[i] = 1.0f; /* FrameBuffer::Clear, FrameBuffer.cpp:97-103 */
        f.win[i] = -1;
    }
    for (size_t i = 0; i < npad; i++)
        f.l0[i] = f.l1[i] = 0.0f;
    run_parallel(&f, out, 0, ntiles, P->threads);
    run_parallel(&f, out, 1, P->height, P->threads);

    out->fragments = 0;
    for (long long k = 0; k < ntiles; k++) out->fragments += f.tileFrags[k];
    out->raster_tris = f.nrt;
    out->bin_refs = f.refStart[ntiles];
    {
        long long clipped = 0;
        for (long long i = 0; i < M->nt; i++)
        {
            const uint32_t* ix = M->indices + 3 * (size_t)i;
            const unsigned c0 = clip_code(f.proj[ix[0]]), c1 = clip_code(f.proj[ix[1]]), c2 = clip_code(f.proj[ix[2]]);
            if ((c0 | c1 | c2) && !(c0 & c1 & c2)) clipped++;
        }
        out->clipped_input_tris = clipped;
    }
    rc = 0;
done:
    free(f.proj); free(f.rv); free(f.rt); free(f.refStart); free(f.refs);
    free(f.depth); free(f.win); free(f.l0); free(f.l1); free(f.tileFrags);
    if (f.tex)
    {
        for (int i = 0; i < P->num_textures; i++) free(f.tex[i].texels);
        free(f.tex);
    }
    return rc;
}
