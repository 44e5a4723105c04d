// Device-side arithmetic of the EDXRaster pipeline.
//
// Integer work is int32 with wraparound (the reference's SSE paddd / pmulld);
// it is written through uint32_t so no signed overflow is relied upon.  Every
// float operation that feeds coverage, depth or the winning triangle uses the
// explicit round-to-nearest intrinsics (__fmul_rn, __fadd_rn, __fdiv_rn ...)
// so the compiler can never contract or reorder it; the library is also
// built with -fmad=false.
#pragma once

#include "edxr_internal.h"

namespace edxr {

__device__ __forceinline__ int wadd(int a, int b) { return (int)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int wsub(int a, int b) { return (int)((uint32_t)a - (uint32_t)b); }
__device__ __forceinline__ int wmul(int a, int b) { return (int)((uint32_t)a * (uint32_t)b); }

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// Matrix::TransformPoint(Vector4(p, 1)) (Shader.h:45): row i is summed left to
// right, ((m0*x + m1*y) + m2*z) + m3*1.
__device__ __forceinline__ float4 xform_point4(const float* M, float x, float y, float z)
{
    float o[4];
#pragma unroll
    for (int i = 0; i < 4; i++)
    {
        float s = fmul(M[i * 4 + 0], x);
        s = fadd(s, fmul(M[i * 4 + 1], y));
        s = fadd(s, fmul(M[i * 4 + 2], z));
        s = fadd(s, fmul(M[i * 4 + 3], 1.0f));
        o[i] = s;
    }
    return make_float4(o[0], o[1], o[2], o[3]);
}

// Matrix::TransformPoint(Vector3) with the raster matrix (RasterTriangle.h:30-32):
// homogeneous divide only when the resulting w is not exactly one.
__device__ __forceinline__ void xform_point3(const float* M, float x, float y, float z, float& ox, float& oy)
{
    float o[4];
#pragma unroll
    for (int i = 0; i < 4; i++)
    {
        float s = fmul(M[i * 4 + 0], x);
        s = fadd(s, fmul(M[i * 4 + 1], y));
        s = fadd(s, fmul(M[i * 4 + 2], z));
        s = fadd(s, M[i * 4 + 3]);
        o[i] = s;
    }
    if (o[3] == 1.0f)
    {
        ox = o[0];
        oy = o[1];
    }
    else
    {
        ox = fdiv(o[0], o[3]);
        oy = fdiv(o[1], o[3]);
    }
}

// v.x = a.x * 16.0 (RasterTriangle.h:35-40): the reference multiplies in
// double and truncates toward zero; NaN and out-of-range give INT_MIN, as the
// x86 cvttsd2si conversion does.  Scaling by 16 is exact in float as well
// (no float reaches overflow by it, and subnormals scale exactly), so the
// float product holds the same value as the double one and its truncation is
// the same integer; no FP64 instruction is needed.  The bounds are the int32
// range: every float >= -2^31 is > -2^31 - 1.
__device__ __forceinline__ int snap16(float f)
{
    const float s = fmul(f, 16.0f);
    if (!(s >= -2147483648.0f && s < 2147483648.0f))
        return (int)0x80000000;
    return __float2int_rz(s);
}

// Clipper::ComputeClipCode (Clipper.h:48-68).
enum : uint32_t { kLeft = 1, kRight = 2, kBottom = 4, kTop = 8, kNear = 16, kFar = 32 };

__device__ __forceinline__ uint32_t clip_code(float4 v)
{
    uint32_t c = 0;
    if (v.x < -v.w) c |= kLeft;
    if (v.x > v.w) c |= kRight;
    if (v.y < -v.w) c |= kBottom;
    if (v.y > v.w) c |= kTop;
    if (v.z > v.w) c |= kFar;
    if (v.z < 0.0f) c |= kNear;
    return c;
}

__device__ __forceinline__ bool plane_inside(int plane, float4 v)
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

// t of the intersection, exactly as written in Clipper.h:241-276.
__device__ __forceinline__ float plane_t(int plane, float4 a, float4 b)
{
    switch (plane)
    {
    case 0: return fdiv(fadd(a.w, a.x), fsub(fadd(a.x, a.w), fadd(b.x, b.w)));
    case 1: return fdiv(fadd(-a.w, a.x), fsub(fsub(a.x, a.w), fsub(b.x, b.w)));
    case 2: return fdiv(fadd(a.w, a.y), fsub(fadd(a.y, a.w), fadd(b.y, b.w)));
    case 3: return fdiv(fadd(-a.w, a.y), fsub(fsub(a.y, a.w), fsub(b.y, b.w)));
    case 4: return fdiv(fadd(-a.w, a.z), fsub(fsub(a.z, a.w), fsub(b.z, b.w)));
    default: return fdiv(a.z, fsub(a.z, b.z));
    }
}

struct PolyVert
{
    float4 p;
    float w0, w1, w2;
};

// Intersection vertex (Clipper.h:210-214,221-224): v0*(1-t) + v1*t, snapped
// onto the plane, and the clip weights blended with the same factors.
__device__ __forceinline__ PolyVert plane_cut(int plane, const PolyVert& a, const PolyVert& b)
{
    const float t = plane_t(plane, a.p, b.p);
    const float s = fsub(1.0f, t);
    PolyVert r;
    r.p.x = fadd(fmul(a.p.x, s), fmul(b.p.x, t));
    r.p.y = fadd(fmul(a.p.y, s), fmul(b.p.y, t));
    r.p.z = fadd(fmul(a.p.z, s), fmul(b.p.z, t));
    r.p.w = fadd(fmul(a.p.w, s), fmul(b.p.w, t));
    switch (plane)
    {
    case 0: r.p.x = -r.p.w; break;
    case 1: r.p.x = r.p.w; break;
    case 2: r.p.y = -r.p.w; break;
    case 3: r.p.y = r.p.w; break;
    case 4: r.p.z = r.p.w; break;
    default: r.p.z = 0.0f; break;
    }
    r.w0 = fadd(fmul(a.w0, s), fmul(b.w0, t));
    r.w1 = fadd(fmul(a.w1, s), fmul(b.w1, t));
    r.w2 = fadd(fmul(a.w2, s), fmul(b.w2, t));
    return r;
}

// Reject / accept corner of one edge from the sign of B / float(C) and of C
// (RasterTriangle.h:66-150); packed as rej | acc << 2.  The quotient of two
// converted ints is never rounded to zero and keeps the sign of B*C, so
// "slope >= 0" is decided exactly without a division: true when B == 0 and
// C != 0 (+-0), when C == 0 and B > 0 (+inf), or when B and C have the same
// sign; 0/0 is NaN and compares false.
__device__ __forceinline__ uint32_t corner_code(int B, int C)
{
    const bool cpos = C >= 0;
    const bool slope_nonneg = (B == 0) ? (C != 0) : ((B > 0) == cpos);
    uint32_t rej, acc;
    if (slope_nonneg) { rej = cpos ? 3u : 0u; acc = cpos ? 0u : 3u; }
    else { rej = cpos ? 2u : 1u; acc = cpos ? 1u : 2u; }
    return rej | (acc << 2);
}

// Per-vertex part of the setup: projection (x, y, z) / w with the
// correctly rounded 1 / w, the raster transform and the snap to the 1/16
// subpixel grid.
__device__ __forceinline__ void project_vertex(const FrameDesc& f, float4 c, int& vx, int& vy, float& z, float& iw)
{
    const float invW = __frcp_rn(c.w);  // == 1.0f / w, correctly rounded
    const float hx = fmul(c.x, invW), hy = fmul(c.y, invW), hz = fmul(c.z, invW);
    float rx, ry;
    xform_point3(f.raster, hx, hy, hz, rx, ry);
    vx = snap16(rx);
    vy = snap16(ry);
    z = hz;
    iw = invW;
}

// Per-triangle part of the setup from the three projected vertices: edge
// coefficients, determinant (culls det <= 0), 1 / det and the corners.
__device__ __forceinline__ bool setup_projected(const int* vx, const int* vy, const float* zp, const float* iw, RTri& t)
{
    const int B0 = wsub(vy[0], vy[1]), C0 = wsub(vx[1], vx[0]);
    const int B1 = wsub(vy[1], vy[2]), C1 = wsub(vx[2], vx[1]);
    const int B2 = wsub(vy[2], vy[0]), C2 = wsub(vx[0], vx[2]);
    const int det = wsub(wmul(C2, B1), wmul(C1, B2));
    if (det <= 0)
        return false;
    t.v0x = vx[0]; t.v0y = vy[0];
    t.v1x = vx[1]; t.v1y = vy[1];
    t.v2x = vx[2]; t.v2y = vy[2];
    t.invDet = __frcp_rn(__int2float_rn(det));
    t.z0 = zp[0]; t.z1 = zp[1]; t.z2 = zp[2];
    t.invW0 = iw[0]; t.invW1 = iw[1]; t.invW2 = iw[2];
    t.meta = corner_code(B0, C0) | (corner_code(B1, C1) << 4) | (corner_code(B2, C2) << 8);
    return true;
}

// RasterTriangle::Setup (RasterTriangle.h:27-153) for three clip-space
// vertices, plus the post-pass of Renderer.cpp:139-147 (invW = 1/w,
// z *= invW).  Returns false for back-facing or degenerate triangles.
__device__ __forceinline__ bool setup_triangle(const FrameDesc& f, float4 c0, float4 c1, float4 c2, RTri& t)
{
    int vx[3], vy[3];
    float zp[3], iw[3];
    project_vertex(f, c0, vx[0], vy[0], zp[0], iw[0]);
    project_vertex(f, c1, vx[1], vy[1], zp[1], iw[1]);
    project_vertex(f, c2, vx[2], vy[2], zp[2], iw[2]);
    return setup_projected(vx, vy, zp, iw, t);
}

// Edge coefficients B, C of a setup triangle (RasterTriangle.h:42-47).
struct Edges
{
    int B[3], C[3];
    int vx[3], vy[3];
};

__device__ __forceinline__ Edges tri_edges(const RTri& t)
{
    Edges e;
    e.vx[0] = t.v0x; e.vy[0] = t.v0y;
    e.vx[1] = t.v1x; e.vy[1] = t.v1y;
    e.vx[2] = t.v2x; e.vy[2] = t.v2y;
#pragma unroll
    for (int k = 0; k < 3; k++)
    {
        const int n = (k + 1) % 3;
        e.B[k] = wsub(e.vy[k], e.vy[n]);
        e.C[k] = wsub(e.vx[n], e.vx[k]);
    }
    return e;
}

// Top-left bias of the scalar edge functions used by binning and the coarse
// step (RasterTriangle.h:155-158): 0 on a top-left edge, else -1.
__device__ __forceinline__ int tl_scalar(int ax, int ay, int bx, int by)
{
    return ((by > ay) || (ay == by && ax > bx)) ? 0 : -1;
}
// Bias of the 4-wide pixel edge functions (RasterTriangle.h:296-299): the
// comparison mask converts to -1 on a top-left edge, else 0.
__device__ __forceinline__ int tl_pixel(int ax, int ay, int bx, int by)
{
    return ((by > ay) || (ay == by && ax > bx)) ? -1 : 0;
}

// EdgeFunc0..2 (RasterTriangle.h:160-171).
__device__ __forceinline__ int edge_scalar(const Edges& e, int k, int px, int py)
{
    const int n = (k + 1) % 3;
    return wadd(wadd(wmul(e.B[k], wsub(px, e.vx[k])), wmul(e.C[k], wsub(py, e.vy[k]))),
                tl_scalar(e.vx[k], e.vy[k], e.vx[n], e.vy[n]));
}

// Lane q of GenStepVectors (RasterTriangle.h:192-255) for one edge: from
// the tested corner (cx, cy) = (corner & 1, corner >> 1) to the same corner
// of quadrant (qx, qy) = (q & 1, q >> 1), (qx - cx) * B + (qy - cy) * C, in
// steps of stepSize = blockSize << 3 = 256 (blockSize = 32).  The table of
// the reference lists exactly these sums; int32 arithmetic wraps the same
// way in either order.
__device__ __forceinline__ int step_lane(uint32_t corner, int B, int C, int q)
{
    const int dx = (q & 1) - (int)(corner & 1), dy = (q >> 1) - (int)(corner >> 1);
    return wmul(256, wadd(wmul(dx, B), wmul(dy, C)));
}

// Per-triangle binning geometry.
// True when no edge function of t can wrap around int32 at a sample within
// 64 pixels of its bounding box: every |B*dx + C*dy| there is at most
// 2 * (extent + 1024)^2 in 1/16-pixel units.  Such a triangle covers a pixel
// centre only inside its closed outline, so only centres inside the
// vertices' bounding box can be covered.
__device__ __forceinline__ bool wrap_free(const RTri& t)
{
    const int minx = min(t.v0x, min(t.v1x, t.v2x)), maxx = max(t.v0x, max(t.v1x, t.v2x));
    const int miny = min(t.v0y, min(t.v1y, t.v2y)), maxy = max(t.v0y, max(t.v1y, t.v2y));
    const float wx = (float)maxx - (float)minx + 1024.0f, wy = (float)maxy - (float)miny + 1024.0f;
    return 2.0f * wx * wy < 1073741824.0f;
}

// Pixels whose centre (16 * p + 8) lies in the closed interval [lo, hi] of
// 1/16-pixel coordinates: [ceil((lo - 8) / 16), floor((hi - 8) / 16)].
__device__ __forceinline__ int centre_lo(int lo) { return (int)(((long long)lo + 7) >> 4); }
__device__ __forceinline__ int centre_hi(int hi) { return (int)(((long long)hi - 8) >> 4); }

struct BinGeom
{
    int bbx0, bbx1, bby0, bby1;      // pixel bounding box (v >> 4)
    int cx0, cx1, cy0, cy1;          // pixels whose centre is inside the vertices' bounding box
    int t32x0, t32x1, t32y0, t32y1;  // reference 32x32 tile range (Renderer.cpp:168-171)
    int t16x0, t16x1, t16y0, t16y1;  // candidate 16x16 tiles
    bool small;                      // Renderer.cpp:173
};

__device__ __forceinline__ BinGeom bin_geom(const RTri& t, const FrameDesc& f)
{
    BinGeom g;
    const int minx = min(t.v0x, min(t.v1x, t.v2x)), maxx = max(t.v0x, max(t.v1x, t.v2x));
    const int miny = min(t.v0y, min(t.v1y, t.v2y)), maxy = max(t.v0y, max(t.v1y, t.v2y));
    g.bbx0 = minx >> 4; g.bbx1 = maxx >> 4;
    g.bby0 = miny >> 4; g.bby1 = maxy >> 4;
    g.cx0 = centre_lo(minx); g.cx1 = centre_hi(maxx);
    g.cy0 = centre_lo(miny); g.cy1 = centre_hi(maxy);
    g.t32x0 = max(0, minx >> 9); g.t32x1 = min(f.tdx32 - 1, maxx >> 9);
    g.t32y0 = max(0, miny >> 9); g.t32y1 = min(f.tdy32 - 1, maxy >> 9);
    g.small = (g.t32x1 - g.t32x0 < 2) && (g.t32y1 - g.t32y0 < 2);
    g.t16x0 = g.t32x0 * 2; g.t16x1 = min(f.tdx - 1, g.t32x1 * 2 + 1);
    g.t16y0 = g.t32y0 * 2; g.t16y1 = min(f.tdy - 1, g.t32y1 * 2 + 1);
    return g;
}

// Does the fine-raster region of the reference (the quad-aligned bounding
// box, Rasterizer.h:132-140) touch an on-screen pixel of 16x16 tile (tx, ty)?
__device__ __forceinline__ bool fine_region_hits(const BinGeom& g, const FrameDesc& f, int tx, int ty)
{
    const int x0 = max(tx * kTileSize, g.bbx0 & ~1);
    const int x1 = min(min(tx * kTileSize + kTileSize - 1, f.width - 1), g.bbx1 | 1);
    const int y0 = max(ty * kTileSize, g.bby0 & ~1);
    const int y1 = min(min(ty * kTileSize + kTileSize - 1, f.height - 1), g.bby1 | 1);
    return x0 <= x1 && y0 <= y1;
}

// The reference's treatment of the four 16x16 quadrants of 32x32 tile
// (T32x, T32y) for a triangle that is not small: per quadrant 0 (not
// rasterized), kDecisionAccept (TrivialAcceptTriangle: every pixel is
// depth-tested) or kDecisionFine (FineRasterize: edge test per pixel inside
// the quad-aligned bounding box), 2 bits each at quadrant q = (tx & 1) +
// 2 * (ty & 1), zero for quadrants off the screen's tile range.  Follows the
// binning of Renderer.cpp:173-227, RasterizeTile (Renderer.cpp:248-270) and
// CoarseRasterize (Rasterizer.h:32-111) with their int32 wraparound.
__device__ __forceinline__ uint32_t quad_decisions(const RTri& t, const Edges& e, const BinGeom& g,
                                                   const FrameDesc& f, int T32x, int T32y)
{
    const int shift = kRefTileLog2 + 4;
    uint32_t rej[3], acc[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
    {
        rej[k] = (t.meta >> (4 * k)) & 3u;
        acc[k] = (t.meta >> (4 * k + 2)) & 3u;
    }
#pragma unroll
    for (int k = 0; k < 3; k++)
    {
        const int cx = (T32x + (int)(rej[k] & 1)) << shift;
        const int cy = (T32y + (int)(rej[k] >> 1)) << shift;
        if (edge_scalar(e, k, cx, cy) < 0)
            return 0;
    }
    bool accE[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
    {
        const int cx = (T32x + (int)(acc[k] & 1)) << shift;
        const int cy = (T32y + (int)(acc[k] >> 1)) << shift;
        accE[k] = edge_scalar(e, k, cx, cy) >= 0;
    }
    // quadrants inside the screen's 16x16 tile range
    uint32_t on = 0;
#pragma unroll
    for (int q = 0; q < 4; q++)
        if (2 * T32x + (q & 1) <= g.t16x1 && 2 * T32y + (q >> 1) <= g.t16y1)
            on |= 1u << q;
    uint32_t out = 0;
    if (accE[0] && accE[1] && accE[2])
    {
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (on & (1u << q))
                out |= kDecisionAccept << (2 * q);
        return out;
    }
    int re[3], ae[3];
    if (f.hierarchical)
    {
        const int baseX = (T32x << kRefTileLog2) << 4, baseY = (T32y << kRefTileLog2) << 4;
        const int span = (32 << 4) - 1;
#pragma unroll
        for (int k = 0; k < 3; k++)
        {
            re[k] = edge_scalar(e, k, baseX + (int)(rej[k] & 1) * span, baseY + (int)(rej[k] >> 1) * span);
            ae[k] = edge_scalar(e, k, baseX + (int)(acc[k] & 1) * span, baseY + (int)(acc[k] >> 1) * span);
        }
    }
#pragma unroll
    for (int q = 0; q < 4; q++)
    {
        if (!(on & (1u << q)))
            continue;
        const int tx = 2 * T32x + (q & 1), ty = 2 * T32y + (q >> 1);
        uint32_t d = kDecisionFine;
        if (f.hierarchical)
        {
            // CoarseRasterize on the 32x32 tile, quadrant q
            bool rejected = false, all = true;
#pragma unroll
            for (int k = 0; k < 3; k++)
            {
                rejected = rejected || wadd(re[k], step_lane(rej[k], e.B[k], e.C[k], q)) < 0;
                // IntSSE(EDX_INFINITY): an edge accepted on the whole tile always accepts
                all = all && (accE[k] || wadd(ae[k], step_lane(acc[k], e.B[k], e.C[k], q)) >= 0);
            }
            if (rejected)
                d = 0;
            else if (all)
                d = kDecisionAccept;
        }
        if (d == kDecisionFine && !fine_region_hits(g, f, tx, ty))
            d = 0;
        out |= d << (2 * q);
    }
    return out;
}

// Monotone key of a depth value: -0 and +0 share a key, float order is
// preserved for all non-NaN values.
__device__ __forceinline__ uint32_t depth_key(float d)
{
    const uint32_t u = __float_as_uint(d == 0.0f ? 0.0f : d);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
// Shading arithmetic (not part of the bit-exact pipeline): fused
// multiply-adds, one rounding each.
__device__ __forceinline__ float dot3(float3 a, float3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ float3 lerp3(float b0, float3 a, float b1, float3 b, float b2, float3 c)
{
    return f3(fmaf(b0, a.x, fmaf(b1, b.x, b2 * c.x)), fmaf(b0, a.y, fmaf(b1, b.y, b2 * c.y)),
              fmaf(b0, a.z, fmaf(b1, b.z, b2 * c.z)));
}
// 1/sqrt(x) from the hardware estimate refined by one Newton step (relative
// error a few 1e-8, well inside the 1e-5 colour tolerance).
__device__ __forceinline__ float rsqrt_nr(float x)
{
    const float y = rsqrtf(x);
    return y * fmaf(-0.5f * x * y, y, 1.5f);
}
__device__ __forceinline__ float3 normalize3(float3 v)
{
    const float inv = rsqrt_nr(dot3(v, v));
    return f3(v.x * inv, v.y * inv, v.z * inv);
}
__device__ __forceinline__ float3 ld3(const char* base, uint32_t stride, uint32_t i, float dflt)
{
    if (!base)
        return f3(dflt, dflt, dflt);
    const float* p = reinterpret_cast<const float*>(base + (size_t)i * stride);
    return f3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}

// Per-pixel shading inputs of a triangle: its three vertices' position,
// normal and albedo (after clipping) in object space.
struct ShadeVerts
{
    float3 p[3], n[3], a[3];
};

// Attributes of the raster vertices of triangle t (Clipper.h:138-151 for the
// vertices the clipper created: weight.x*a0 + weight.y*a1 + weight.z*a2).
__device__ __forceinline__ ShadeVerts shade_verts(const FrameDesc& f, const RTri& t, const ClipPoly* polys)
{
    const uint32_t tri = t.order >> 4;
    const uint32_t i0 = __ldg(f.indices + 3 * (size_t)tri + 0);
    const uint32_t i1 = __ldg(f.indices + 3 * (size_t)tri + 1);
    const uint32_t i2 = __ldg(f.indices + 3 * (size_t)tri + 2);
    float3 sp[3] = { ld3(f.positions, f.pos_stride, i0, 0.f), ld3(f.positions, f.pos_stride, i1, 0.f), ld3(f.positions, f.pos_stride, i2, 0.f) };
    float3 sn[3] = { ld3(f.normals, f.nrm_stride, i0, 0.f), ld3(f.normals, f.nrm_stride, i1, 0.f), ld3(f.normals, f.nrm_stride, i2, 0.f) };
    float3 sa[3] = { ld3(f.albedo, f.alb_stride, i0, 1.f), ld3(f.albedo, f.alb_stride, i1, 1.f), ld3(f.albedo, f.alb_stride, i2, 1.f) };
    ShadeVerts v;
    if (t.poly == kUnclipped)
    {
#pragma unroll
        for (int k = 0; k < 3; k++) { v.p[k] = sp[k]; v.n[k] = sn[k]; v.a[k] = sa[k]; }
        return v;
    }
    const ClipPoly& P = polys[t.poly >> 4];
    const int fk = (int)(t.poly & 15u);
    const int pv[3] = { 0, fk - 1, fk };
#pragma unroll
    for (int k = 0; k < 3; k++)
    {
        const float w0 = P.w[pv[k]][0], w1 = P.w[pv[k]][1], w2 = P.w[pv[k]][2];
        v.p[k] = f3(fadd(fadd(fmul(w0, sp[0].x), fmul(w1, sp[1].x)), fmul(w2, sp[2].x)),
                    fadd(fadd(fmul(w0, sp[0].y), fmul(w1, sp[1].y)), fmul(w2, sp[2].y)),
                    fadd(fadd(fmul(w0, sp[0].z), fmul(w1, sp[1].z)), fmul(w2, sp[2].z)));
        v.n[k] = f3(fadd(fadd(fmul(w0, sn[0].x), fmul(w1, sn[1].x)), fmul(w2, sn[2].x)),
                    fadd(fadd(fmul(w0, sn[0].y), fmul(w1, sn[1].y)), fmul(w2, sn[2].y)),
                    fadd(fadd(fmul(w0, sn[0].z), fmul(w1, sn[1].z)), fmul(w2, sn[2].z)));
        v.a[k] = f3(fadd(fadd(fmul(w0, sa[0].x), fmul(w1, sa[1].x)), fmul(w2, sa[2].x)),
                    fadd(fadd(fmul(w0, sa[0].y), fmul(w1, sa[1].y)), fmul(w2, sa[2].y)),
                    fadd(fadd(fmul(w0, sa[0].z), fmul(w1, sa[1].z)), fmul(w2, sa[2].z)));
    }
    return v;
}

// The shading model on interpolated attributes (Shader.h:249-281 structure):
//   N = normalize(n), L = light, E = normalize(eye - p), H = normalize(L + E)
//   diffuse = (max(N.L, 0) + 0.2) * 3/pi
//   BLINN_PHONG:           albedo*diffuse + ks*max(N.H, 0)^shininess
//   BLINN_PHONG_REFERENCE: diffuse + ks*(N.H)^shininess
//   LAMBERTIAN_ALBEDO:     albedo*diffuse
//   LAMBERTIAN:            diffuse
__device__ __forceinline__ float3 shade_model(const FrameDesc& f, float3 P, float3 Nraw, float3 A)
{
    const float3 N = normalize3(Nraw);
    const float3 L = f3(f.light[0], f.light[1], f.light[2]);
    const float nl = fmaxf(dot3(L, N), 0.0f);
    const float diffuse = (nl + 0.2f) * 0.954929658551372f;  // 3/pi
    float spec = 0.0f;
    if (f.ps_kind <= 1)
    {
        const float3 E = normalize3(f3(f.eye[0] - P.x, f.eye[1] - P.y, f.eye[2] - P.z));
        const float3 H = normalize3(f3(L.x + E.x, L.y + E.y, L.z + E.z));
        float nh = dot3(N, H);
        if (f.ps_kind == 0)
            nh = fmaxf(nh, 0.0f);
        // nh^shininess as 2^(shininess log2 nh) (nh is clamped to >= 0 here:
        // log2 0 = -inf gives 0; the unclamped reference shader shades in FP64)
        spec = f.ks * exp2f(f.shininess * log2f(nh));
    }
    switch (f.ps_kind)
    {
    case 0: return f3(fmaf(A.x, diffuse, spec), fmaf(A.y, diffuse, spec), fmaf(A.z, diffuse, spec));
    case 1: return f3(diffuse + spec, diffuse + spec, diffuse + spec);
    case 2:
    case 4: return f3(A.x * diffuse, A.y * diffuse, A.z * diffuse);
    default: return f3(diffuse, diffuse, diffuse);
    }
}

// ---------------------------------------------------------------------------
// Texture sampling (Texture2D::Sample(uv, differentials) of the textured
// Lambertian shader, Shader.h:226-239).  EDXUtil's sampler is not part of the
// reference; this build's contract, restated operation for operation in the
// oracle: coordinates repeat; texel (x, y) covers [x, x+1) x [y, y+1) in
// texel units; nearest and bilinear sample level 0; trilinear takes the
// level of detail 0.5 log2(max |d|^2) of the two differentials in texels and
// blends the bilinear samples of the two levels around it; anisotropic Nx
// takes n = min(N, ceil(major / minor)) trilinear probes along the longer
// differential, at the level of detail of major / n, and averages them.
__device__ __forceinline__ float wrap01(float u) { return u - floorf(u); }
__device__ __forceinline__ float lerpf(float a, float b, float t) { return fmaf(t, b - a, a); }
__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t)
{
    return make_float4(lerpf(a.x, b.x, t), lerpf(a.y, b.y, t), lerpf(a.z, b.z, t), lerpf(a.w, b.w, t));
}

struct TexLevel
{
    const float4* texels;
    int w, h;
};

__device__ __forceinline__ TexLevel tex_level(const FrameDesc& f, const TexDesc& d, int level)
{
    uint64_t off = d.base;
    int w = (int)d.width, h = (int)d.height;
    for (int l = 0; l < level; l++)
    {
        off += (uint64_t)w * h;
        w = max(1, w >> 1);
        h = max(1, h >> 1);
    }
    return { f.texels + off, w, h };
}

__device__ __forceinline__ float4 tex_fetch(const TexLevel& L, int x, int y)
{
    x %= L.w;
    if (x < 0) x += L.w;
    y %= L.h;
    if (y < 0) y += L.h;
    return __ldg(L.texels + (size_t)y * L.w + x);
}

__device__ __forceinline__ float4 tex_bilinear(const TexLevel& L, float u, float v)
{
    const float fx = wrap01(u) * (float)L.w - 0.5f, fy = wrap01(v) * (float)L.h - 0.5f;
    const float x0 = floorf(fx), y0 = floorf(fy);
    const float tx = fx - x0, ty = fy - y0;
    const int ix = (int)x0, iy = (int)y0;
    const float4 a = lerp4(tex_fetch(L, ix, iy), tex_fetch(L, ix + 1, iy), tx);
    const float4 b = lerp4(tex_fetch(L, ix, iy + 1), tex_fetch(L, ix + 1, iy + 1), tx);
    return lerp4(a, b, ty);
}

__device__ __forceinline__ float4 tex_trilinear(const FrameDesc& f, const TexDesc& d, float u, float v, float lod)
{
    lod = fminf(fmaxf(lod, 0.0f), (float)(d.levels - 1));
    const int l0 = (int)floorf(lod);
    const float t = lod - (float)l0;
    const float4 c0 = tex_bilinear(tex_level(f, d, l0), u, v);
    if (t == 0.0f)
        return c0;
    return lerp4(c0, tex_bilinear(tex_level(f, d, min(l0 + 1, (int)d.levels - 1)), u, v), t);
}

__device__ __forceinline__ float4 sample_texture(const FrameDesc& f, const TexDesc& d, float u, float v, float2 d0,
                                                 float2 d1)
{
    switch (f.tex_filter)
    {
    case 0:
    {
        const TexLevel L = tex_level(f, d, 0);
        const int x = min((int)floorf(wrap01(u) * (float)L.w), L.w - 1);
        const int y = min((int)floorf(wrap01(v) * (float)L.h), L.h - 1);
        return tex_fetch(L, x, y);
    }
    case 1: return tex_bilinear(tex_level(f, d, 0), u, v);
    default: break;
    }
    const float ax = d0.x * (float)d.width, ay = d0.y * (float)d.height;
    const float bx = d1.x * (float)d.width, by = d1.y * (float)d.height;
    const float r0 = fmaf(ax, ax, ay * ay), r1 = fmaf(bx, bx, by * by);
    if (f.tex_filter == 2)
    {
        const float r = fmaxf(r0, r1);
        return tex_trilinear(f, d, u, v, r > 1.0f ? 0.5f * log2f(r) : 0.0f);
    }
    const int N = f.tex_filter == 3 ? 4 : (f.tex_filter == 4 ? 8 : 16);
    const float l0 = sqrtf(r0), l1 = sqrtf(r1);
    const float major = fmaxf(l0, l1), minor = fminf(l0, l1);
    const int n = major <= 0.0f ? 1 : (minor <= 0.0f ? N : min(N, (int)ceilf(major / minor)));
    const float2 axis = l0 >= l1 ? d0 : d1;
    const float m = major / (float)n;
    const float lod = m > 1.0f ? log2f(m) : 0.0f;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = 0; i < n; i++)
    {
        const float s = ((float)i + 0.5f) / (float)n - 0.5f;
        const float4 c = tex_trilinear(f, d, fmaf(axis.x, s, u), fmaf(axis.y, s, v), lod);
        acc = make_float4(acc.x + c.x, acc.y + c.y, acc.z + c.z, acc.w + c.w);
    }
    const float inv = 1.0f / (float)n;
    return make_float4(acc.x * inv, acc.y * inv, acc.z * inv, acc.w * inv);
}

// Perspective-correct barycentrics of triangle t at the centre of pixel
// (px, py) (TriangleSSE::CalcBarycentricCoord, RasterTriangle.h:333-337, then
// Fragment::Interpolate, Shader.h:150-158).
__device__ __forceinline__ float3 persp_bary(const RTri& t, int px, int py)
{
    const int cx = (px << 4) + 8, cy = (py << 4) + 8;
    const Edges e = tri_edges(t);
    const int n1 = wadd(wmul(e.B[1], wsub(cx, t.v2x)), wmul(e.C[1], wsub(cy, t.v2y)));
    const int n2 = wadd(wmul(e.B[2], wsub(cx, t.v2x)), wmul(e.C[2], wsub(cy, t.v2y)));
    float b0 = fmul(__int2float_rn(n1), t.invDet), b1 = fmul(__int2float_rn(n2), t.invDet);
    float b2 = fsub(fsub(1.0f, b0), b1);
    b0 = fmul(b0, t.invW0);
    b1 = fmul(b1, t.invW1);
    b2 = fmul(b2, t.invW2);
    const float invB = fdiv(1.0f, fadd(fadd(b0, b1), b2));
    b0 = fmul(b0, invB);
    b1 = fmul(b1, invB);
    return f3(b0, b1, fsub(fsub(1.0f, b0), b1));
}

// Albedo of the textured Lambertian shader at pixel (px, py) of triangle t:
// the texture coordinate interpolated there, and the differentials of the
// pixel's 2x2 quad (LambertianAlbedoPixelShader, Shader.h:226-228: lane 1
// minus lane 0 and lane 2 minus lane 0, the quad's top-left pixel being
// lane 0), all from t's perspective-correct barycentrics.
// (Out of line, and handed the record's address in global memory, so that a
// caller's copy of it can stay in registers.)
static __device__ __noinline__ float3 texture_albedo(const FrameDesc& f, const RTri* tg, const ClipPoly* polys, int px,
                                                    int py)
{
    const RTri t = *tg;
    const uint32_t tri = t.order >> 4;
    const uint32_t slot = f.tex_ids ? __ldg(f.tex_ids + tri) : 0u;
    if (slot >= f.num_textures || !f.uvs)
        return f3(1.0f, 1.0f, 1.0f);
    float2 uv[3];
    {
        const uint32_t i0 = __ldg(f.indices + 3 * (size_t)tri + 0);
        const uint32_t i1 = __ldg(f.indices + 3 * (size_t)tri + 1);
        const uint32_t i2 = __ldg(f.indices + 3 * (size_t)tri + 2);
        const float* p0 = reinterpret_cast<const float*>(f.uvs + (size_t)i0 * f.uv_stride);
        const float* p1 = reinterpret_cast<const float*>(f.uvs + (size_t)i1 * f.uv_stride);
        const float* p2 = reinterpret_cast<const float*>(f.uvs + (size_t)i2 * f.uv_stride);
        const float2 s[3] = { make_float2(__ldg(p0), __ldg(p0 + 1)), make_float2(__ldg(p1), __ldg(p1 + 1)),
                              make_float2(__ldg(p2), __ldg(p2 + 1)) };
        if (t.poly == kUnclipped)
        {
            uv[0] = s[0]; uv[1] = s[1]; uv[2] = s[2];
        }
        else
        {
            const ClipPoly& P = polys[t.poly >> 4];
            const int fk = (int)(t.poly & 15u);
            const int pv[3] = { 0, fk - 1, fk };
#pragma unroll
            for (int k = 0; k < 3; k++)
            {
                const float w0 = P.w[pv[k]][0], w1 = P.w[pv[k]][1], w2 = P.w[pv[k]][2];
                uv[k] = make_float2(fadd(fadd(fmul(w0, s[0].x), fmul(w1, s[1].x)), fmul(w2, s[2].x)),
                                    fadd(fadd(fmul(w0, s[0].y), fmul(w1, s[1].y)), fmul(w2, s[2].y)));
            }
        }
    }
    auto uv_at = [&](int x, int y) {
        const float3 b = persp_bary(t, x, y);
        return make_float2(fmaf(b.x, uv[0].x, fmaf(b.y, uv[1].x, b.z * uv[2].x)),
                           fmaf(b.x, uv[0].y, fmaf(b.y, uv[1].y, b.z * uv[2].y)));
    };
    const int qx = px & ~1, qy = py & ~1;
    const float2 q0 = uv_at(qx, qy), q1 = uv_at(qx + 1, qy), q2 = uv_at(qx, qy + 1);
    const float2 here = (px == qx && py == qy) ? q0 : (py == qy ? q1 : (px == qx ? q2 : uv_at(px, py)));
    const float4 c = sample_texture(f, f.textures[slot], here.x, here.y, make_float2(q1.x - q0.x, q1.y - q0.y),
                                    make_float2(q2.x - q0.x, q2.y - q0.y));
    return f3(c.x, c.y, c.z);
}

// BlinnPhongPixelShader as written (ks = 3, exponent 200, no clamp) amplifies
// the error of N.H by ks*s*x^(s-1) = 600: FP32 unit vectors cannot hold N.H
// to the ~5e-9 that 1e-5 of colour needs, so this shader interpolates and
// shades in FP64.
static __device__ __noinline__ float3 shade_fragment_fp64(const FrameDesc& f, const RTri* tg, const ClipPoly* polys,
                                                   float l0, float l1)
{
    const RTri t = *tg;
    double b0 = l0, b1 = l1;
    double b2 = 1.0 - b0 - b1;
    b0 *= (double)t.invW0;
    b1 *= (double)t.invW1;
    b2 *= (double)t.invW2;
    const double s = 1.0 / (b0 + b1 + b2);
    b0 *= s;
    b1 *= s;
    b2 = 1.0 - b0 - b1;
    const ShadeVerts v = shade_verts(f, t, polys);
    double P[3], N[3];
    const float* vp[3] = { &v.p[0].x, &v.p[1].x, &v.p[2].x };
    const float* vn[3] = { &v.n[0].x, &v.n[1].x, &v.n[2].x };
    for (int q = 0; q < 3; q++)
    {
        P[q] = b0 * vp[0][q] + b1 * vp[1][q] + b2 * vp[2][q];
        N[q] = b0 * vn[0][q] + b1 * vn[1][q] + b2 * vn[2][q];
    }
    double inv = 1.0 / sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
    for (int q = 0; q < 3; q++) N[q] *= inv;
    double L[3] = { f.light_raw[0], f.light_raw[1], f.light_raw[2] };
    inv = 1.0 / sqrt(L[0] * L[0] + L[1] * L[1] + L[2] * L[2]);
    for (int q = 0; q < 3; q++) L[q] *= inv;
    double nl = L[0] * N[0] + L[1] * N[1] + L[2] * N[2];
    if (nl < 0.0) nl = 0.0;
    const double diffuse = (nl + 0.2) * 3.0 / 3.14159265358979323846;
    double E[3] = { f.eye_d[0] - P[0], f.eye_d[1] - P[1], f.eye_d[2] - P[2] };
    inv = 1.0 / sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
    double H[3];
    for (int q = 0; q < 3; q++) H[q] = L[q] + E[q] * inv;
    inv = 1.0 / sqrt(H[0] * H[0] + H[1] * H[1] + H[2] * H[2]);
    const double nh = (N[0] * H[0] + N[1] * H[1] + N[2] * H[2]) * inv;
    const float c = (float)(diffuse + (double)f.ks * pow(nh, (double)f.shininess));
    return f3(c, c, c);
}

// Fragment::Interpolate (Shader.h:142-170) from the fragment's barycentrics,
// then the shading model.
// t is the record at tg (global memory).
__device__ __forceinline__ float3 shade_fragment(const FrameDesc& f, const RTri& t, const RTri* tg,
                                                 const ClipPoly* polys, float l0, float l1, int px, int py)
{
    if (f.ps_kind == 1)
        return shade_fragment_fp64(f, tg, polys, l0, l1);
    float b0 = l0, b1 = l1;
    float b2 = fsub(fsub(1.0f, b0), b1);
    b0 = fmul(b0, t.invW0);
    b1 = fmul(b1, t.invW1);
    b2 = fmul(b2, t.invW2);
    const float invB = __frcp_rn(fadd(fadd(b0, b1), b2));
    b0 = fmul(b0, invB);
    b1 = fmul(b1, invB);
    b2 = fsub(fsub(1.0f, b0), b1);
    const ShadeVerts v = shade_verts(f, t, polys);
    const float3 P = lerp3(b0, v.p[0], b1, v.p[1], b2, v.p[2]);
    const float3 N = lerp3(b0, v.n[0], b1, v.n[1], b2, v.n[2]);
    const float3 A = f.ps_kind == 4 ? texture_albedo(f, tg, polys, px, py) : lerp3(b0, v.a[0], b1, v.a[1], b2, v.a[2]);
    return shade_model(f, P, N, A);
}

// Frame owning output pixel i (binary search over pix_base).
__device__ __forceinline__ uint32_t frame_of_pixel64(const FrameDesc* frames, uint32_t n, uint64_t p)
{
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi)
    {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (frames[mid].pix_base <= p) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Frame owning flattened index i, by binary search over a monotone base
// field (tri_base or tile_base) of the frame array.
template <typename Get>
__device__ __forceinline__ uint32_t find_frame(const FrameDesc* frames, uint32_t n, uint32_t i, Get get)
{
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi)
    {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (get(frames[mid]) <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

}  // namespace edxr
