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

__device__ __forceinline__ uint32_t frame_of_pixel(const FrameDesc* frames, uint32_t n, uint64_t p)
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
    // The solve cancels heavily (a_k, c_k are the small projected distances of
    // the vertices from the pixel centre, each a difference of O(1) terms), so
    // the clip coordinates, the pixel centre and the solve run in FP64; the
    // result is rounded to float once.  FP64 is the slow unit of this GPU:
    // the products are fused explicitly (fma) and S is inverted once.
    double X[3], Y[3], Wd[3], ac[3], cc[3], bt[3];
    const float* M = f.mvp;
    for (int k = 0; k < 3; k++)
    {
        const double x = s.p[k].x, y = s.p[k].y, z = s.p[k].z;
        X[k] = fma((double)M[0], x, fma((double)M[1], y, fma((double)M[2], z, (double)M[3])));
        Y[k] = fma((double)M[4], x, fma((double)M[5], y, fma((double)M[6], z, (double)M[7])));
        Wd[k] = fma((double)M[12], x, fma((double)M[13], y, fma((double)M[14], z, (double)M[15])));
        s.X[k] = (float)X[k];
        s.Y[k] = (float)Y[k];
        s.W[k] = (float)Wd[k];
    }
    const double rx = (double)px + 0.5, ry = (double)py + 0.5;
    const double* R = f.ndc_from_raster_d;
    const double u = fma(R[0], rx, fma(R[1], ry, R[2]));
    const double v = fma(R[3], rx, fma(R[4], ry, R[5]));
    s.u = (float)u;
    s.v = (float)v;
    for (int k = 0; k < 3; k++)
    {
        ac[k] = fma(-u, Wd[k], X[k]);
        cc[k] = fma(-v, Wd[k], Y[k]);
        s.ac[k] = (float)ac[k];
        s.cc[k] = (float)cc[k];
    }
    bt[0] = fma(ac[1], cc[2], -(ac[2] * cc[1]));
    bt[1] = fma(ac[2], cc[0], -(ac[0] * cc[2]));
    bt[2] = fma(ac[0], cc[1], -(ac[1] * cc[0]));
    const double S = bt[0] + bt[1] + bt[2];
    if (!(S != 0.0))
        return false;
    s.S = (float)S;
    const double invS = 1.0 / S;
    for (int k = 0; k < 3; k++)
    {
        s.bt[k] = (float)bt[k];
        s.b[k] = (float)(bt[k] * invS);
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
    const FrameDesc& f = a.frames[frame_of_pixel(a.frames, a.num_frames, i)];
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
        const FrameDesc& f = a.frames[frame_of_pixel(a.frames, a.num_frames, i)];
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
