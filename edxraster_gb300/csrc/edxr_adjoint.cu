// Differentiable form: shading of the visible surface with visibility held
// fixed, and its hand-written adjoint.
//
// Forward (k_shade_visible), per pixel with a winning triangle t (the
// triangle-id buffer of the last pass):
//   clip_k = MVP (p_k, 1) for t's three input vertices (Shader.h:45)
//   (u, v) = NDC of the pixel centre; a_k = X_k - u W_k, c_k = Y_k - v W_k
//   b = (a x c) / sum(a x c)   perspective-correct barycentrics of the point
//                              of t's plane that projects to the pixel centre
//                              (the same weights Fragment::Interpolate forms,
//                              Shader.h:142-170, without the 1/16 snap, so they
//                              are smooth in the vertex positions; clipping
//                              does not change them)
//   P, N, A = sum b_k (p_k, n_k, albedo_k); colour = shading model (the same
//   one the raster kernel uses, edxr_device.cuh shade_model).
// Adjoint (k_backward): the same recomputation, then reverse-mode through
// the shading model, the interpolation, the barycentric solve and the MVP
// transform.  Per-vertex gradients are accumulated with float atomics; the
// light, ks and shininess gradients are reduced per block and accumulated in
// double.  Nothing per pixel is stored between the passes.
#include <cuda_runtime.h>

#include "edxr_device.cuh"

namespace edxr {

namespace {

constexpr int kThreads = 256;

// Frame of flattened output pixel p: one division when the pass's frames
// share one resolution (tiles_per_frame set: the batched pass), else a
// search over the frames' first pixels.
__device__ __forceinline__ uint32_t frame_of_pixel(const PassArgs& a, uint64_t p)
{
    if (a.tiles_per_frame)
    {
        const uint64_t per_frame = a.total_pixels / a.num_frames;
        return a.total_pixels <= 0xFFFFFFFFull ? (uint32_t)p / (uint32_t)per_frame : (uint32_t)(p / per_frame);
    }
    const FrameDesc* frames = a.frames;
    const uint32_t n = a.num_frames;
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi)
    {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (frames[mid].pix_base <= p) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

struct V3
{
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return { x, y, z }; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return { s * a.x, s * a.y, s * a.z }; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len(V3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ V3 ld(const char* base, uint32_t stride, uint32_t i, float dflt)
{
    if (!base)
        return v3(dflt, dflt, dflt);
    const float* p = reinterpret_cast<const float*>(base + (size_t)i * stride);
    return v3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}
// gradient of normalize(x) applied to dy: (dy - y (y . dy)) / |x|
__device__ __forceinline__ V3 normalize_grad(V3 y, float lenx, V3 dy) { return (1.0f / lenx) * (dy - dot(y, dy) * y); }

// Float pairs: the value hi + lo, |lo| <= ulp(hi) / 2.
struct FF
{
    float hi, lo;
};
// a * b exactly, as a pair (needs the product rounded once: the library is
// built without contraction, and fmaf gives the exact remainder).
__device__ __forceinline__ FF two_prod(float a, float b)
{
    const float p = a * b;
    return { p, fmaf(a, b, -p) };
}
// a + b exactly, as a pair.
__device__ __forceinline__ FF two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return { s, (a - (s - bb)) + (b - bb) };
}
__device__ __forceinline__ FF quick_two_sum(float a, float b)  // |a| >= |b|
{
    const float s = a + b;
    return { s, b - (s - a) };
}
__device__ __forceinline__ FF ff_add(FF x, FF y)
{
    const FF s = two_sum(x.hi, y.hi);
    return quick_two_sum(s.hi, s.lo + (x.lo + y.lo));
}
__device__ __forceinline__ FF ff_sub(FF x, FF y) { return ff_add(x, { -y.hi, -y.lo }); }
__device__ __forceinline__ FF ff_mul(FF x, FF y)
{
    const FF p = two_prod(x.hi, y.hi);
    return quick_two_sum(p.hi, p.lo + (x.hi * y.lo + x.lo * y.hi));
}
__device__ __forceinline__ FF ff_mul_f(FF x, float y)
{
    const FF p = two_prod(x.hi, y);
    return quick_two_sum(p.hi, p.lo + x.lo * y);
}
// m0 x + m1 y + m2 z + m3 as a pair.
__device__ __forceinline__ FF ff_dot4(float m0, float m1, float m2, float m3, float x, float y, float z)
{
    return ff_add(ff_add(two_prod(m0, x), two_prod(m1, y)), ff_add(two_prod(m2, z), { m3, 0.0f }));
}
// Everything the forward computes for one pixel, kept for the adjoint.
struct PixelState
{
    uint32_t vi[3];
    V3 p[3], n[3], a[3];
    float X[3], Y[3], W[3];
    float ac[3], cc[3];
    float bt[3], S, b[3];
    float u, v;
    V3 P, Nraw, A;
};

__device__ __forceinline__ bool pixel_forward(const FrameDesc& f, const DiffMesh& m, uint32_t tri, int px, int py,
                                              PixelState& s)
{
    if (tri >= m.nt)
        return false;
    for (int k = 0; k < 3; k++)
    {
        s.vi[k] = __ldg(m.indices + 3 * (size_t)tri + k);
        if (s.vi[k] >= m.nv)
            return false;
        s.p[k] = ld(m.positions, m.pos_stride, s.vi[k], 0.0f);
        s.n[k] = ld(m.normals, m.nrm_stride, s.vi[k], 0.0f);
        s.a[k] = ld(m.albedo, m.alb_stride, s.vi[k], 1.0f);
    }
    // The solve cancels heavily: a_k, c_k are the small projected distances of
    // the vertices from the pixel centre, each a difference of O(1) terms.
    // The clip coordinates and the pixel centre are therefore carried as
    // float pairs (hi + lo, about 48 bits; error-free products and sums,
    // Dekker 1971 / Knuth), and so are a_k, c_k, the cross products and their
    // sum, each rounded to float once: FP32 arithmetic throughout, accurate
    // to a few float ulps of the results, without the FP64 unit (slow on
    // this GPU).
    const float* M = f.mvp;
    FF X[3], Y[3], Wd[3];
    for (int k = 0; k < 3; k++)
    {
        const float x = s.p[k].x, y = s.p[k].y, z = s.p[k].z;
        X[k] = ff_dot4(M[0], M[1], M[2], M[3], x, y, z);
        Y[k] = ff_dot4(M[4], M[5], M[6], M[7], x, y, z);
        Wd[k] = ff_dot4(M[12], M[13], M[14], M[15], x, y, z);
        s.X[k] = X[k].hi + X[k].lo;
        s.Y[k] = Y[k].hi + Y[k].lo;
        s.W[k] = Wd[k].hi + Wd[k].lo;
    }
    const float rx = (float)px + 0.5f, ry = (float)py + 0.5f;  // exact
    const float* Rh = f.ndc_from_raster;
    const float* Rl = f.ndc_from_raster_lo;
    const FF u = ff_add(ff_add(ff_mul_f({ Rh[0], Rl[0] }, rx), ff_mul_f({ Rh[1], Rl[1] }, ry)), { Rh[2], Rl[2] });
    const FF v = ff_add(ff_add(ff_mul_f({ Rh[3], Rl[3] }, rx), ff_mul_f({ Rh[4], Rl[4] }, ry)), { Rh[5], Rl[5] });
    s.u = u.hi + u.lo;
    s.v = v.hi + v.lo;
    FF ac[3], cc[3];
    for (int k = 0; k < 3; k++)
    {
        ac[k] = ff_sub(X[k], ff_mul(u, Wd[k]));
        cc[k] = ff_sub(Y[k], ff_mul(v, Wd[k]));
        s.ac[k] = ac[k].hi + ac[k].lo;
        s.cc[k] = cc[k].hi + cc[k].lo;
    }
    // the cross products and their sum stay pairs too: near an edge, or on a
    // thin triangle, they cancel again
    FF bt[3];
    bt[0] = ff_sub(ff_mul(ac[1], cc[2]), ff_mul(ac[2], cc[1]));
    bt[1] = ff_sub(ff_mul(ac[2], cc[0]), ff_mul(ac[0], cc[2]));
    bt[2] = ff_sub(ff_mul(ac[0], cc[1]), ff_mul(ac[1], cc[0]));
    const FF Sf = ff_add(ff_add(bt[0], bt[1]), bt[2]);
    const float S = Sf.hi + Sf.lo;
    if (!(S != 0.0f) || !(fabsf(S) < 3.0e38f))
        return false;
    s.S = S;
    for (int k = 0; k < 3; k++)
    {
        s.bt[k] = bt[k].hi + bt[k].lo;
        s.b[k] = s.bt[k] / S;
    }
    s.P = s.b[0] * s.p[0] + s.b[1] * s.p[1] + s.b[2] * s.p[2];
    s.Nraw = s.b[0] * s.n[0] + s.b[1] * s.n[1] + s.b[2] * s.n[2];
    s.A = s.b[0] * s.a[0] + s.b[1] * s.a[1] + s.b[2] * s.a[2];
    return true;
}

// Shading model on (P, N, A); flags of the pixel shader kinds of edxr.h.
struct ShadeTerms
{
    V3 Nn, L, E, H;
    float nlen, llen, elen, hlen;
    float nl, nh, nhc, powv, diffuse, spec;
    bool albedo, specular, clamp;
};

// Light, ks and shininess in effect for frame f.
struct Shading
{
    float light[3], ks, shininess;
};
__device__ __forceinline__ Shading shading_of(const FrameDesc& f, const DiffMesh& m)
{
    if (m.override_shading)
        return { { m.light[0], m.light[1], m.light[2] }, m.ks, m.shininess };
    return { { f.light_raw[0], f.light_raw[1], f.light_raw[2] }, f.ks, f.shininess };
}

__device__ __forceinline__ V3 shade_forward(const FrameDesc& f, const Shading& sh, const PixelState& s,
                                            ShadeTerms& t)
{
    t.albedo = (f.ps_kind == 0 || f.ps_kind == 2);
    t.specular = (f.ps_kind <= 1);
    t.clamp = (f.ps_kind == 0);
    t.nlen = len(s.Nraw);
    t.Nn = (1.0f / t.nlen) * s.Nraw;
    const V3 l = v3(sh.light[0], sh.light[1], sh.light[2]);
    t.llen = len(l);
    t.L = (1.0f / t.llen) * l;
    t.nl = dot(t.L, t.Nn);
    t.diffuse = (fmaxf(t.nl, 0.0f) + 0.2f) * 0.954929658551372f;
    t.spec = 0.0f;
    if (t.specular)
    {
        const V3 Er = v3(f.eye[0], f.eye[1], f.eye[2]) - s.P;
        t.elen = len(Er);
        t.E = (1.0f / t.elen) * Er;
        const V3 Hr = t.L + t.E;
        t.hlen = len(Hr);
        t.H = (1.0f / t.hlen) * Hr;
        t.nh = dot(t.Nn, t.H);
        t.nhc = t.clamp ? fmaxf(t.nh, 0.0f) : t.nh;
        t.powv = powf(t.nhc, sh.shininess);
        t.spec = sh.ks * t.powv;
    }
    if (t.albedo)
        return v3(s.A.x * t.diffuse + t.spec, s.A.y * t.diffuse + t.spec, s.A.z * t.diffuse + t.spec);
    return v3(t.diffuse + t.spec, t.diffuse + t.spec, t.diffuse + t.spec);
}

__global__ void __launch_bounds__(kThreads) k_shade_visible(PassArgs a, uint64_t total, DiffMesh m, float4* out)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total)
        return;
    const FrameDesc& f = a.frames[frame_of_pixel(a, i)];
    const uint64_t local = i - f.pix_base;
    const int px = (int)(local % (uint32_t)f.width), py = (int)(local / (uint32_t)f.width);
    const uint32_t tri = a.tri_id[i];
    PixelState s;
    if (tri == kNoTriangle || !pixel_forward(f, m, tri, px, py, s))
    {
        out[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    ShadeTerms t;
    const V3 c = shade_forward(f, shading_of(f, m), s, t);
    out[i] = make_float4(c.x, c.y, c.z, 1.0f);
}

__device__ __forceinline__ void add3(float* g, uint32_t v, V3 d)
{
    if (!g)
        return;
    atomicAdd(g + 3 * (size_t)v + 0, d.x);
    atomicAdd(g + 3 * (size_t)v + 1, d.y);
    atomicAdd(g + 3 * (size_t)v + 2, d.z);
}

__global__ void __launch_bounds__(kThreads) k_backward(PassArgs a, uint64_t total, DiffMesh m, const float4* grad,
                                                       DiffGrads g)
{
    __shared__ float red[5 * (kThreads / 32)];
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    V3 dl = v3(0.f, 0.f, 0.f);
    float dks = 0.0f, dshin = 0.0f;
    if (i < total)
    {
        const FrameDesc& f = a.frames[frame_of_pixel(a, i)];
        const uint64_t local = i - f.pix_base;
        const int px = (int)(local % (uint32_t)f.width), py = (int)(local / (uint32_t)f.width);
        const uint32_t tri = a.tri_id[i];
        PixelState s;
        if (tri != kNoTriangle && pixel_forward(f, m, tri, px, py, s))
        {
            ShadeTerms t;
            const Shading sh = shading_of(f, m);
            shade_forward(f, sh, s, t);
            const float4 gc = grad[i];
            const V3 gcol = v3(gc.x, gc.y, gc.z);
            // colour = (albedo ? A * diffuse : diffuse) + spec
            const V3 dA = t.albedo ? t.diffuse * gcol : v3(0.f, 0.f, 0.f);
            const float ddiff = t.albedo ? dot(gcol, s.A) : (gcol.x + gcol.y + gcol.z);
            const float dspec = t.specular ? (gcol.x + gcol.y + gcol.z) : 0.0f;
            V3 dNn = v3(0.f, 0.f, 0.f), dL = v3(0.f, 0.f, 0.f), dP = v3(0.f, 0.f, 0.f);
            // diffuse = (max(nl, 0) + 0.2) * 3/pi
            const float dnl = (t.nl > 0.0f) ? ddiff * 0.954929658551372f : 0.0f;
            dL = dL + dnl * t.Nn;
            dNn = dNn + dnl * t.L;
            if (t.specular)
            {
                // spec = ks * nhc^s
                dks = dspec * t.powv;
                if (t.nhc > 0.0f)
                    dshin = dspec * sh.ks * t.powv * logf(t.nhc);
                float dnh = 0.0f;
                if (!t.clamp || t.nh > 0.0f)
                    dnh = (sh.shininess == 0.0f) ? 0.0f
                                                 : dspec * sh.ks * sh.shininess * powf(t.nhc, sh.shininess - 1.0f);
                dNn = dNn + dnh * t.H;
                const V3 dH = dnh * t.Nn;
                const V3 dHr = normalize_grad(t.H, t.hlen, dH);  // H = normalize(L + E)
                dL = dL + dHr;
                const V3 dEr = normalize_grad(t.E, t.elen, dHr);  // E = normalize(eye - P)
                dP = dP - dEr;
            }
            const V3 dNraw = normalize_grad(t.Nn, t.nlen, dNn);
            dl = normalize_grad(t.L, t.llen, dL);
            // P, N, A = sum b_k (p_k, n_k, a_k)
            float db[3];
            for (int k = 0; k < 3; k++)
            {
                add3(g.albedo, s.vi[k], s.b[k] * dA);
                add3(g.normals, s.vi[k], s.b[k] * dNraw);
                db[k] = dot(dP, s.p[k]) + dot(dNraw, s.n[k]) + dot(dA, s.a[k]);
            }
            // b = bt / S
            const float bdb = s.b[0] * db[0] + s.b[1] * db[1] + s.b[2] * db[2];
            float dbt[3];
            for (int k = 0; k < 3; k++)
                dbt[k] = (db[k] - bdb) / s.S;
            // bt = a x c
            float dac[3] = { 0.f, 0.f, 0.f }, dcc[3] = { 0.f, 0.f, 0.f };
            dac[1] += dbt[0] * s.cc[2]; dcc[2] += dbt[0] * s.ac[1]; dac[2] -= dbt[0] * s.cc[1]; dcc[1] -= dbt[0] * s.ac[2];
            dac[2] += dbt[1] * s.cc[0]; dcc[0] += dbt[1] * s.ac[2]; dac[0] -= dbt[1] * s.cc[2]; dcc[2] -= dbt[1] * s.ac[0];
            dac[0] += dbt[2] * s.cc[1]; dcc[1] += dbt[2] * s.ac[0]; dac[1] -= dbt[2] * s.cc[0]; dcc[0] -= dbt[2] * s.ac[1];
            // a_k = X_k - u W_k, c_k = Y_k - v W_k, (X, Y, W) = rows 0, 1, 3 of MVP (p, 1)
            if (g.positions)
                for (int k = 0; k < 3; k++)
                {
                    const float dX = dac[k], dY = dcc[k], dW = -s.u * dac[k] - s.v * dcc[k];
                    const float* M = f.mvp;
                    V3 dp = v3(M[0] * dX + M[4] * dY + M[12] * dW, M[1] * dX + M[5] * dY + M[13] * dW,
                               M[2] * dX + M[6] * dY + M[14] * dW);
                    dp = dp + s.b[k] * dP;
                    add3(g.positions, s.vi[k], dp);
                }
        }
    }
    // block-reduce the five global gradients together (one barrier),
    // accumulate in double
    float vals[5] = { dl.x, dl.y, dl.z, dks, dshin };
#pragma unroll
    for (int q = 0; q < 5; q++)
        for (int o = 16; o > 0; o >>= 1)
            vals[q] += __shfl_down_sync(0xffffffffu, vals[q], o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < 5; q++)
            red[q * (kThreads / 32) + warp] = vals[q];
    __syncthreads();
    if (warp == 0)
    {
#pragma unroll
        for (int q = 0; q < 5; q++)
        {
            float r = lane < kThreads / 32 ? red[q * (kThreads / 32) + lane] : 0.0f;
            for (int o = 16; o > 0; o >>= 1)
                r += __shfl_down_sync(0xffffffffu, r, o);
            if (lane == 0 && r != 0.0f)
                atomicAdd(g.scratch + q, (double)r);
        }
    }
}

__global__ void k_zero_globals(double* scratch)
{
    if (threadIdx.x < 5)
        scratch[threadIdx.x] = 0.0;
}

__global__ void k_finish_globals(DiffGrads g)
{
    if (threadIdx.x != 0)
        return;
    if (g.light)
        for (int q = 0; q < 3; q++)
            g.light[q] += (float)g.scratch[q];
    if (g.ks)
        g.ks[0] += (float)g.scratch[3];
    if (g.shininess)
        g.shininess[0] += (float)g.scratch[4];
}

}  // namespace

cudaError_t launch_shade_visible(const PassArgs& a, uint64_t total, const DiffMesh& m, float4* out, cudaStream_t s)
{
    if (total)
        k_shade_visible<<<(unsigned)((total + kThreads - 1) / kThreads), kThreads, 0, s>>>(a, total, m, out);
    return cudaGetLastError();
}

cudaError_t launch_backward(const PassArgs& a, uint64_t total, const DiffMesh& m, const float4* grad,
                            const DiffGrads& g, cudaStream_t s)
{
    k_zero_globals<<<1, 32, 0, s>>>(g.scratch);
    if (total)
        k_backward<<<(unsigned)((total + kThreads - 1) / kThreads), kThreads, 0, s>>>(a, total, m, grad, g);
    k_finish_globals<<<1, 32, 0, s>>>(g);
    return cudaGetLastError();
}

}  // namespace edxr
