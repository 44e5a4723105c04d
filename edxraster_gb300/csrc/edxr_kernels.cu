// CUDA kernels of the EDXRaster GB300 pipeline (sm_103a).
//
// One pass renders any number of frames (a frame = one mesh seen by one
// camera); the plain path is a pass of one frame.  Stages:
//   k_clear        zero the per-tile counters and work queues
//   k_vertex       clip = MVP * (p, 1) per (frame, vertex)     Shader.h:40-49
//   k_setup        clip codes, clipping, fixed-point setup      Clipper.h:71-189,
//                  and the post-pass, per input triangle        RasterTriangle.h:27-153
//   k_bin*         (triangle, 16x16 tile) decisions, counted,   Renderer.cpp:161-229
//                  scanned and scattered into per-tile bins
//   k_raster       persistent tiles: coverage, depth test and   Renderer.cpp:248-270,
//                  winner per pixel                             Rasterizer.h:32-415,
//                                                               FrameBuffer.cpp:54-68
//   k_shade        deferred shading of the winner; one write    Renderer.cpp:272-350
//                  of colour, depth and triangle id per pixel
#include <cuda_runtime.h>

#include "edxr_device.cuh"

namespace edxr {

constexpr int kRasterThreads = 256;    // one thread per pixel of a 16x16 tile
constexpr int kScanItems = 4;
constexpr int kScanThreads = 1024;
constexpr int kScanBlock = kScanItems * kScanThreads;

// -------------------------------------------------------------------------
__global__ void k_clear(PassArgs a)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= a.total_tiles; i += stride)
    {
        a.tile_count[i] = 0;
        a.tile_cursor[i] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x < 8)
        a.counters[threadIdx.x] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        a.status->overflow = 0;
        a.status->error = 0;
        a.status->bins_needed = 0;
        a.status->raster_tris = 0;
        a.status->clipped_polys = 0;
        a.status->big_tris = 0;
    }
}

// -------------------------------------------------------------------------
// Vertex stage: one thread per (frame, vertex).
__global__ void __launch_bounds__(256) k_vertex(PassArgs a)
{
    const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= a.total_vertices)
        return;
    const uint32_t fi = find_frame(a.frames, a.num_frames, gi, [](const FrameDesc& f) { return f.vtx_base; });
    const FrameDesc& f = a.frames[fi];
    const uint32_t v = gi - f.vtx_base;
    const float* p = reinterpret_cast<const float*>(f.positions + (size_t)v * f.pos_stride);
    a.clip[gi] = xform_point4(f.mvp, __ldg(p), __ldg(p + 1), __ldg(p + 2));
}

// -------------------------------------------------------------------------
// Clipping + setup: one thread per input triangle.  Surviving triangles are
// appended with a warp-aggregated atomic; each carries its submission order.
__device__ __forceinline__ void clip_triangle(const FrameDesc& f, float4 c0, float4 c1, float4 c2,
                                              uint32_t planes, PolyVert* poly, int& n, float4* vclip)
{
    poly[0] = { c0, 1.f, 0.f, 0.f };
    poly[1] = { c1, 0.f, 1.f, 0.f };
    poly[2] = { c2, 0.f, 0.f, 1.f };
    n = clip_polygon(poly, planes);
    // Clipper.h:121-152: a vertex whose weight is exactly one on a source
    // vertex is that source vertex (position and attributes); others are new.
    const float4 src[3] = { c0, c1, c2 };
    for (int j = 0; j < n; j++)
    {
        int s = -1;
        if (poly[j].w0 == 1.0f) s = 0;
        else if (poly[j].w1 == 1.0f) s = 1;
        else if (poly[j].w2 == 1.0f) s = 2;
        if (s >= 0)
        {
            poly[j].w0 = (s == 0) ? 1.f : 0.f;
            poly[j].w1 = (s == 1) ? 1.f : 0.f;
            poly[j].w2 = (s == 2) ? 1.f : 0.f;
            vclip[j] = src[s];
        }
        else
            vclip[j] = poly[j].p;
    }
}

// Appends n raster triangles for this lane with one atomic per warp; returns
// the lane's first slot.  Every lane of the warp must call it.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, int n)
{
    const uint32_t lane = threadIdx.x & 31;
    int incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && total > 0)
        base = atomicAdd(counter, (uint32_t)total);
    return __shfl_sync(0xffffffffu, base, 31) + (uint32_t)(incl - n);
}

// Setup of the triangles that need no clipping (all clip codes zero), one
// thread per input triangle; triangles that straddle a clip plane are queued
// for k_clip, triangles outside one plane are dropped (Clipper.h:103-109).
__global__ void __launch_bounds__(256) k_setup(PassArgs a)
{
    const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t fi = 0, tri = 0;
    int nOut = 0;
    RTri t;
    if (gi < a.total_tris)
    {
        fi = find_frame(a.frames, a.num_frames, gi, [](const FrameDesc& f) { return f.tri_base; });
        const FrameDesc& f = a.frames[fi];
        tri = gi - f.tri_base;
        const uint32_t i0 = __ldg(f.indices + 3 * (size_t)tri);
        const uint32_t i1 = __ldg(f.indices + 3 * (size_t)tri + 1);
        const uint32_t i2 = __ldg(f.indices + 3 * (size_t)tri + 2);
        if (i0 >= f.nv || i1 >= f.nv || i2 >= f.nv)
        {
            // device-resident index buffers are checked here instead of on the host
            atomicOr(&a.status->error, 1u);  // EDXR_ERR_INVALID_ARG
        }
        else
        {
            const float4 c0 = a.clip[f.vtx_base + i0];
            const float4 c1 = a.clip[f.vtx_base + i1];
            const float4 c2 = a.clip[f.vtx_base + i2];
            const uint32_t k0 = clip_code(c0), k1 = clip_code(c1), k2 = clip_code(c2);
            if ((k0 | k1 | k2) == 0)
                nOut = setup_triangle(f, c0, c1, c2, t) ? 1 : 0;
            else if (!(k0 & k1 & k2))
            {
                const uint32_t q = atomicAdd(&a.counters[4], 1u);
                if (q < a.poly_capacity)
                    a.clip_list[q] = gi;
            }
        }
    }
    const uint32_t base = warp_append(&a.counters[0], nOut);
    if (gi < a.total_tris)
        a.tri_first[gi] = (nOut && base < a.rtri_capacity) ? base : kNoTriangle;  // k_clip sets clipped ones
    if (nOut == 0)
        return;
    if (base >= a.rtri_capacity)
    {
        atomicOr(&a.status->overflow, 2u);
        return;
    }
    t.order = tri << 4;
    t.meta |= fi << 12;
    t.poly = kUnclipped;
    a.rtris[base] = t;
}

// Clipping of the queued triangles (Clipper.h:107-171): Sutherland-Hodgman,
// fan triangulation, setup of each fan triangle.  Grid-stride over the queue.
__global__ void __launch_bounds__(128) k_clip(PassArgs a)
{
    const uint32_t nq = min(*(volatile uint32_t*)&a.counters[4], a.poly_capacity);
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (nq + stride - 1) / stride;
    for (uint32_t r = 0; r < rounds; r++)
    {
        const uint32_t q = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
        PolyVert poly[kMaxPolygon];
        float4 vc[kMaxPolygon];
        int n = 0, nOut = 0;
        uint32_t gi = 0, fi = 0, tri = 0;
        if (q < nq)
        {
            gi = a.clip_list[q];
            fi = find_frame(a.frames, a.num_frames, gi, [](const FrameDesc& f) { return f.tri_base; });
            const FrameDesc& f = a.frames[fi];
            tri = gi - f.tri_base;
            const float4 c0 = a.clip[f.vtx_base + __ldg(f.indices + 3 * (size_t)tri)];
            const float4 c1 = a.clip[f.vtx_base + __ldg(f.indices + 3 * (size_t)tri + 1)];
            const float4 c2 = a.clip[f.vtx_base + __ldg(f.indices + 3 * (size_t)tri + 2)];
            const uint32_t k0 = clip_code(c0), k1 = clip_code(c1), k2 = clip_code(c2);
            clip_triangle(f, c0, c1, c2, (k0 ^ k1) | (k1 ^ k2) | (k2 ^ k0), poly, n, vc);
            for (int k = 2; k < n; k++)
            {
                RTri tmp;
                nOut += setup_triangle(f, vc[0], vc[k - 1], vc[k], tmp) ? 1 : 0;
            }
        }
        uint32_t out = warp_append(&a.counters[0], nOut);
        if (nOut == 0)
            continue;
        if (out + (uint32_t)nOut > a.rtri_capacity)
        {
            atomicOr(&a.status->overflow, 2u);
            continue;
        }
        const FrameDesc& f = a.frames[fi];
        const uint32_t pi = atomicAdd(&a.counters[1], 1u);
        if (pi >= a.poly_capacity)
        {
            atomicOr(&a.status->overflow, 4u);
            continue;
        }
        ClipPoly& P = a.polys[pi];
        for (int j = 0; j < n; j++)
        {
            P.w[j][0] = poly[j].w0;
            P.w[j][1] = poly[j].w1;
            P.w[j][2] = poly[j].w2;
        }
        P.n = (uint32_t)n;
        // the surviving fan triangles are contiguous and in fan order
        a.tri_first[gi] = out;
        for (int k = 2; k < n; k++)
        {
            RTri tk;
            if (!setup_triangle(f, vc[0], vc[k - 1], vc[k], tk))
                continue;
            tk.order = (tri << 4) | (uint32_t)(k - 2);
            tk.meta |= fi << 12;
            tk.poly = (pi << 4) | (uint32_t)k;
            a.rtris[out++] = tk;
        }
    }
}

// -------------------------------------------------------------------------
// Binning.  Phase 0 counts the non-rejected (triangle, tile) pairs per tile,
// phase 1 writes entries (raster triangle << 2 | decision).  Triangles the
// reference treats as small go through a lean per-thread path whose
// decisions are cheap enough to compute again in phase 1; the others are
// binned by one warp each with the full decision of tile_decision, counted
// and appended to an unsorted list at once (phase 2) and moved into their
// bins by k_bin_move after the scan.
//
// bin_emit counts or writes one entry for `tile` (decision d; nothing when
// d is 0).  Neighbouring triangles of a warp often land in the same tile:
// lanes with equal tiles share one atomic, issued by the lowest lane.
template <int Phase>
__device__ __forceinline__ void bin_emit(const PassArgs& a, uint32_t ri, uint32_t d, uint32_t tile_in)
{
    const uint32_t act = __activemask();
    const uint32_t tile = d ? tile_in : 0xFFFFFFFFu;
    const uint32_t peers = __match_any_sync(act, tile);
    const uint32_t hits = __ballot_sync(act, d != 0);
    if (!d)
        return;
    const uint32_t lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    if (Phase != 1)
    {
        if ((int)lane == leader)
            atomicAdd(&a.tile_count[tile], (uint32_t)__popc(peers));
    }
    if (Phase == 2)
    {
        const int first = __ffs(hits) - 1;
        uint32_t base = 0;
        if ((int)lane == first)
            base = atomicAdd(&a.counters[5], (uint32_t)__popc(hits));
        base = __shfl_sync(hits, base, first) + (uint32_t)__popc(hits & ((1u << lane) - 1u));
        if (base < a.bin_capacity)
            a.bin_tmp[base] = make_uint2(tile, (ri << 2) | d);
    }
    if (Phase == 1)
    {
        uint32_t base = 0;
        if ((int)lane == leader)
            base = atomicAdd(&a.tile_cursor[tile], (uint32_t)__popc(peers));
        base = __shfl_sync(peers, base, leader) + (uint32_t)__popc(peers & ((1u << lane) - 1u));
        const uint64_t pos = (uint64_t)a.tile_offset[tile] + base;
        if (pos < a.bin_capacity)
            a.bins[pos] = (ri << 2) | d;
    }
}

template <int Phase>
__device__ __forceinline__ void bin_tile(const PassArgs& a, const FrameDesc& f, uint32_t ri, const RTri& t,
                                         const Edges& e, const BinGeom& g, int tx, int ty)
{
    bin_emit<Phase>(a, ri, tile_decision(t, e, g, f, tx, ty), f.tile_base + (uint32_t)(ty * f.tdx + tx));
}

// Scatter of the decided entries into their bins (after the scan).
__global__ void __launch_bounds__(256) k_bin_move(PassArgs a)
{
    const uint32_t n = *(volatile uint32_t*)&a.counters[5];
    const uint32_t m = (uint32_t)min((uint64_t)n, a.bin_capacity);
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (m + stride - 1) / stride;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t r = 0; r < rounds; r++)
    {
        const uint32_t i = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
        const bool valid = i < m;
        const uint2 e = valid ? a.bin_tmp[i] : make_uint2(0xFFFFFFFFu, 0u);
        const uint32_t peers = __match_any_sync(0xffffffffu, e.x);
        if (!valid)
            continue;
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if ((int)lane == leader)
            base = atomicAdd(&a.tile_cursor[e.x], (uint32_t)__popc(peers));
        base = __shfl_sync(peers, base, leader) + (uint32_t)__popc(peers & ((1u << lane) - 1u));
        const uint64_t pos = (uint64_t)a.tile_offset[e.x] + base;
        if (pos < a.bin_capacity)
            a.bins[pos] = e.y;
    }
}

template <int Phase>
__global__ void __launch_bounds__(256) k_bin(PassArgs a)
{
    const uint32_t n = *(volatile uint32_t*)&a.counters[0];
    const uint32_t nr = min(n, a.rtri_capacity);
    for (uint32_t ri = blockIdx.x * blockDim.x + threadIdx.x; ri < nr; ri += gridDim.x * blockDim.x)
    {
        const RTri t = a.rtris[ri];
        const FrameDesc& f = a.frames[t.meta >> 12];
        const BinGeom g = bin_geom(t, f);
        if (!g.small)
        {
            // bounding box over 2x2 reference tiles: binned warp-cooperatively
            if (Phase == 0)
            {
                const uint32_t b = atomicAdd(&a.counters[2], 1u);
                if (b < a.big_capacity)
                    a.big_list[b] = ri;
            }
            continue;
        }
        // The reference rasterizes a small triangle with FineRasterize in every
        // tile of its range (Renderer.cpp:173-180), so the decision is "fine"
        // exactly where the quad-aligned bounding box meets the screen.
        const int x0 = max(g.bbx0 & ~1, 0), x1 = min(g.bbx1 | 1, f.width - 1);
        const int y0 = max(g.bby0 & ~1, 0), y1 = min(g.bby1 | 1, f.height - 1);
        if (x0 > x1 || y0 > y1)
            continue;
        for (int ty = y0 >> kTileLog2; ty <= (y1 >> kTileLog2); ty++)
            for (int tx = x0 >> kTileLog2; tx <= (x1 >> kTileLog2); tx++)
                bin_emit<Phase>(a, ri, kDecisionFine, f.tile_base + (uint32_t)(ty * f.tdx + tx));
    }
}

// One warp per triangle of the big list; lanes take candidate tiles.  Its
// entries are counted and appended to the unsorted list in one pass.
__global__ void __launch_bounds__(256) k_bin_big(PassArgs a)
{
    const uint32_t nb = min(*(volatile uint32_t*)&a.counters[2], a.big_capacity);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < nb; b += nw)
    {
        const uint32_t ri = a.big_list[b];
        const RTri t = a.rtris[ri];
        const FrameDesc& f = a.frames[t.meta >> 12];
        const BinGeom g = bin_geom(t, f);
        const Edges e = tri_edges(t);
        const int nx = g.t16x1 - g.t16x0 + 1, ny = g.t16y1 - g.t16y0 + 1;
        for (int j = (int)lane; j < nx * ny; j += 32)
            bin_tile<2>(a, f, ri, t, e, g, g.t16x0 + j % nx, g.t16y0 + j / nx);
    }
}

// -------------------------------------------------------------------------
// Exclusive scan of the per-tile counts, each rounded up to a multiple of 4
// entries so every bin starts on a 16-byte boundary.
__device__ __forceinline__ uint32_t padded(uint32_t c) { return (c + 3u) & ~3u; }

__global__ void __launch_bounds__(kScanThreads) k_scan_blocks(PassArgs a, uint32_t* block_sums)
{
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
    uint32_t v[kScanItems], s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
    {
        const uint32_t i = base + k;
        v[k] = (i < a.total_tiles) ? padded(a.tile_count[i]) : 0u;
        s += v[k];
    }
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        uint32_t w = warp_sums[lane];
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= (uint32_t)o) wi += t;
        }
        warp_sums[lane] = wi - w;
        if (lane == 31) block_sums[blockIdx.x] = wi;
    }
    __syncthreads();
    uint32_t run = warp_sums[warp] + incl - s;
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
    {
        const uint32_t i = base + k;
        if (i < a.total_tiles) a.tile_offset[i] = run;
        run += v[k];
    }
}

__global__ void __launch_bounds__(1024) k_scan_spine(uint32_t* block_sums, uint32_t nblocks)
{
    // single block; nblocks <= 1024 * 4
    __shared__ uint32_t warp_sums[32];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t v[4], s = 0;
    for (int k = 0; k < 4; k++)
    {
        const uint32_t i = threadIdx.x * 4 + k;
        v[k] = i < nblocks ? block_sums[i] : 0u;
        s += v[k];
    }
    uint32_t incl = s;
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        const uint32_t w = warp_sums[lane];
        uint32_t wi = w;
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= (uint32_t)o) wi += t;
        }
        warp_sums[lane] = wi - w;
    }
    __syncthreads();
    uint32_t run = warp_sums[warp] + incl - s;
    for (int k = 0; k < 4; k++)
    {
        const uint32_t i = threadIdx.x * 4 + k;
        if (i < nblocks) block_sums[i] = run;  // exclusive
        run += v[k];
    }
    if (threadIdx.x == blockDim.x - 1)
        block_sums[nblocks] = run;  // grand total
}

__global__ void k_scan_add(PassArgs a, const uint32_t* block_sums, uint32_t nblocks)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.total_tiles)
        a.tile_offset[i] += block_sums[i / kScanBlock];
    if (i == 0)
    {
        const uint64_t total = block_sums[nblocks];
        a.tile_offset[a.total_tiles] = (uint32_t)total;
        a.status->bins_needed = total;
        a.status->raster_tris = a.counters[0];
        a.status->clipped_polys = a.counters[1];
        a.status->big_tris = a.counters[2];
        if (a.counters[0] > a.rtri_capacity)
            atomicOr(&a.status->overflow, 2u);
        if (a.counters[1] > a.poly_capacity || a.counters[4] > a.poly_capacity)
            atomicOr(&a.status->overflow, 4u);
        a.status->clipped_polys = max(a.counters[1], a.counters[4]);
        if (total > a.bin_capacity)
            atomicOr(&a.status->overflow, 1u);
        if (a.counters[2] > a.big_capacity)
            atomicOr(&a.status->overflow, 8u);
    }
}

// -------------------------------------------------------------------------
// Raster: persistent blocks take 16x16 tiles from a queue.  The winner of
// the reference's sequential depth test at a pixel is the fragment with the
// smallest key (depth key << 32 | submission rank term): for LEQUAL the last
// fragment with the smallest depth wins, for LESS the first.  Keys can be
// combined in any order, so the bin needs no ordering and two paths can
// share the work:
//  * small entries (quad-aligned region of at most tune.small_region pixels) are
//    rasterized triangle-parallel by the thread that stages them, merging
//    into a shared-memory key per pixel with a 64-bit atomicMin;
//  * the other entries are staged as tile-relative edge equations and
//    rasterized pixel-parallel: warp w owns the 8x4 block at
//    (8*(w&1), 4*(w>>1)), tests 32 staged entries at once (one per lane) for
//    overlap with its block and against its hierarchical depth bound, and
//    walks only the entries whose ballot bit is set.
// The pixel's final key is the minimum of both; its rank (order + 1, 0 when
// nothing passed) goes to the id buffer for k_shade.
struct __align__(16) StagedTri
{
    int A0, D0, K0, A1;    // e0 = A0*lx + D0*ly + K0 (with bias); l1 = A1*lx + D1*ly + K1 (no bias)
    int D1, K1, A2, D2;
    int K2;
    uint32_t flags;        // region lx0|lx1<<5|ly0<<10|ly1<<15, accept<<20, bias1<<21, bias2<<22
    uint32_t rank;         // global rank: (frame tri_base * 16 + order) + 1
    uint32_t pad;
    float invDet, z0, z1, z2;
};

constexpr uint32_t kEmptyRegion = 16u | (16u << 10);  // lx0 = ly0 = 16 > lx1 = ly1 = 0

// Lower bound (as a depth key) of every depth the reference computes for the
// triangle at a pixel it rasterizes, or 0 (never culled) when the triangle is
// large enough for int32 edge values to wrap.  Without wraparound the
// barycentrics of rasterized pixels are within a few ulps of [0, 1], so the
// computed depth is at least min(z) minus a few ulps of the |z| sum.
__device__ __forceinline__ uint32_t zmin_key(const RTri& t)
{
    const int minx = min(t.v0x, min(t.v1x, t.v2x)), maxx = max(t.v0x, max(t.v1x, t.v2x));
    const int miny = min(t.v0y, min(t.v1y, t.v2y)), maxy = max(t.v0y, max(t.v1y, t.v2y));
    const float wx = (float)maxx - (float)minx + 1024.0f, wy = (float)maxy - (float)miny + 1024.0f;
    if (!(2.0f * wx * wy < 1073741824.0f))
        return 0u;
    const float zmin = fminf(t.z0, fminf(t.z1, t.z2));
    const float margin = 2e-6f * (fabsf(t.z0) + fabsf(t.z1) + fabsf(t.z2)) + 1e-30f;
    const float lo = zmin - margin;
    return (lo == lo) ? depth_key(lo) : 0u;
}

// Tile-relative edge equations, barycentric numerators and region of one
// bin entry.
__device__ __forceinline__ void stage_tri(const PassArgs& a, uint32_t entry, uint32_t nr, uint32_t rank_base,
                                          int tileX, int tileY,
                                          StagedTri& s, uint32_t& zkey)
{
    const uint32_t ri = entry >> 2;
    if (ri >= nr)
    {
        // never written by a consistent pass; an empty region keeps it inert
        s.flags = kEmptyRegion;
        zkey = 0xFFFFFFFFu;
        return;
    }
    const bool accept = (entry & 3u) == kDecisionAccept;
    const RTri t = a.rtris[ri];
    const Edges e = tri_edges(t);
    // pixel (lx, ly) of the tile samples at (16*(16*tileX + lx) + 8, ...)
    const int ox = (tileX << 8) + 8, oy = (tileY << 8) + 8;
    int A[3], D[3], K[3], bias[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
    {
        const int n = (k + 1) % 3;
        bias[k] = tl_pixel(e.vx[k], e.vy[k], e.vx[n], e.vy[n]);
        A[k] = wmul(16, e.B[k]);
        D[k] = wmul(16, e.C[k]);
        K[k] = wadd(wmul(e.B[k], wsub(ox, e.vx[k])), wmul(e.C[k], wsub(oy, e.vy[k])));
    }
    s.A0 = A[0]; s.D0 = D[0]; s.K0 = wadd(K[0], bias[0]);
    // the barycentric numerators of RasterTriangle.h:335-336 are edges 1
    // and 2 measured from v2, equal to the unbiased edge values
    s.A1 = A[1]; s.D1 = D[1]; s.K1 = K[1];
    s.A2 = A[2]; s.D2 = D[2]; s.K2 = K[2];
    int lx0 = 0, lx1 = 15, ly0 = 0, ly1 = 15;
    if (!accept)
    {
        const int bbx0 = min(t.v0x, min(t.v1x, t.v2x)) >> 4, bbx1 = max(t.v0x, max(t.v1x, t.v2x)) >> 4;
        const int bby0 = min(t.v0y, min(t.v1y, t.v2y)) >> 4, bby1 = max(t.v0y, max(t.v1y, t.v2y)) >> 4;
        lx0 = max(0, (bbx0 & ~1) - (tileX << 4));
        lx1 = min(15, (bbx1 | 1) - (tileX << 4));
        ly0 = max(0, (bby0 & ~1) - (tileY << 4));
        ly1 = min(15, (bby1 | 1) - (tileY << 4));
        if (lx1 < lx0 || ly1 < ly0) { lx0 = 16; lx1 = 0; ly0 = 16; ly1 = 0; }
    }
    s.flags = (uint32_t)lx0 | ((uint32_t)lx1 << 5) | ((uint32_t)ly0 << 10) | ((uint32_t)ly1 << 15) |
              (accept ? (1u << 20) : 0u) | (bias[1] ? (1u << 21) : 0u) | (bias[2] ? (1u << 22) : 0u);
    s.invDet = t.invDet;
    s.z0 = t.z0; s.z1 = t.z1; s.z2 = t.z2;
    // submission order within the frame, offset by the frame's first input
    // triangle so k_shade can find the record without knowing the frame
    s.rank = rank_base + t.order + 1u;
    zkey = zmin_key(t);
}

// Key of the fragment of staged triangle s at tile pixel (lx, ly), or false
// when the pixel is not covered (FineRasterize's edge test; trivially
// accepted entries skip it) or the depth is NaN (never passes).
__device__ __forceinline__ bool fragment_key(const StagedTri& s, int lx, int ly, bool less, uint64_t& key)
{
    const uint32_t fl = s.flags;
    const int l1 = wadd(wadd(wmul(s.A1, lx), wmul(s.D1, ly)), s.K1);
    const int l2 = wadd(wadd(wmul(s.A2, lx), wmul(s.D2, ly)), s.K2);
    if (!(fl & (1u << 20)))
    {
        const int e0 = wadd(wadd(wmul(s.A0, lx), wmul(s.D0, ly)), s.K0);
        const int e1 = wadd(l1, (fl & (1u << 21)) ? -1 : 0);
        const int e2 = wadd(l2, (fl & (1u << 22)) ? -1 : 0);
        if ((e0 | e1 | e2) < 0)
            return false;
    }
    // TriangleSSE::CalcBarycentricCoord / GetDepth (RasterTriangle.h:324-337)
    const float L0 = fmul(__int2float_rn(l1), s.invDet);
    const float L1 = fmul(__int2float_rn(l2), s.invDet);
    const float L2 = fsub(fsub(1.0f, L0), L1);
    const float d = fadd(fadd(fmul(L0, s.z0), fmul(L1, s.z1)), fmul(L2, s.z2));
    if (d != d)
        return false;
    key = ((uint64_t)depth_key(d) << 32) | (less ? s.rank : ~s.rank);
    return true;
}

template <int MinBlocks, bool SmallPath>
__global__ void __launch_bounds__(kRasterThreads, MinBlocks) k_raster(PassArgs a)
{
    __shared__ StagedTri st[kRasterThreads];
    __shared__ uint32_t s_flags[kRasterThreads];
    __shared__ uint32_t s_zkey[kRasterThreads];
    __shared__ unsigned long long s_key[kRasterThreads];
    __shared__ uint32_t s_tile;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int bx = (int)(warp & 1u) * 8, by = (int)(warp >> 1) * 4;
    const int lx = bx + (int)(lane & 7u), ly = by + (int)(lane >> 3);
    const uint32_t pix = (uint32_t)(ly * 16 + lx);  // this thread's pixel in s_key
    const uint32_t nr = min(*(volatile uint32_t*)&a.counters[0], a.rtri_capacity);
    s_key[pix] = ~0ull;
    for (;;)
    {
        if (threadIdx.x == 0)
            s_tile = atomicAdd(&a.counters[3], 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        __syncthreads();
        if (tile >= a.total_tiles)
            break;
        const uint32_t fi = find_frame(a.frames, a.num_frames, tile, [](const FrameDesc& f) { return f.tile_base; });
        const FrameDesc& f = a.frames[fi];
        const uint32_t lt = tile - f.tile_base;
        const int tileX = (int)(lt % (uint32_t)f.tdx), tileY = (int)(lt / (uint32_t)f.tdx);
        const bool less = f.depth_func == 1;
        uint32_t count = a.tile_count[tile];
        const uint32_t start = a.tile_offset[tile];
        if ((uint64_t)start + count > a.bin_capacity)
            count = 0;  // overflowed frame: rendered again by the host

        // clear depth 1.0 with no triangle: rank term ~0 (LEQUAL) or 0 (LESS)
        uint64_t best = ((uint64_t)0xBF800000u << 32) | (less ? 0u : 0xFFFFFFFFu);
        uint32_t wzmax = 0xBF800000u;  // largest depth key held in this warp's registers

        for (uint32_t c = 0; c < count; c += kRasterThreads)
        {
            const uint32_t m = min((uint32_t)kRasterThreads, count - c);
            if (threadIdx.x < m)
            {
                StagedTri s;
                uint32_t zk;
                stage_tri(a, a.bins[start + c + threadIdx.x], nr, f.tri_base << 4, tileX, tileY, s, zk);
                const uint32_t fl = s.flags;
                const int rx0 = fl & 31, rx1 = (fl >> 5) & 31, ry0 = (fl >> 10) & 31, ry1 = (fl >> 15) & 31;
                const int area = (rx1 - rx0 + 1) * (ry1 - ry0 + 1);
                if (SmallPath && !(fl & (1u << 20)) && rx0 <= rx1 && ry0 <= ry1 && area <= a.tune.small_region)
                {
                    // small: this thread rasterizes the triangle's few pixels
                    for (int y = ry0; y <= ry1; y++)
                        for (int x = rx0; x <= rx1; x++)
                        {
                            uint64_t key;
                            // a plain read first: most fragments of deep overdraw lose
                            if (fragment_key(s, x, y, less, key) && key < s_key[y * 16 + x])
                                atomicMin(&s_key[y * 16 + x], (unsigned long long)key);
                        }
                    s_flags[threadIdx.x] = kEmptyRegion;
                }
                else
                {
                    st[threadIdx.x] = s;
                    s_flags[threadIdx.x] = fl;
                    s_zkey[threadIdx.x] = zk;
                }
            }
            __syncthreads();
            for (uint32_t g = 0; g < m; g += 32)
            {
                const uint32_t jl = g + lane;
                bool hit = false;
                if (jl < m)
                {
                    const uint32_t fl = s_flags[jl];
                    const int lx0 = fl & 31, lx1 = (fl >> 5) & 31, ly0 = (fl >> 10) & 31, ly1 = (fl >> 15) & 31;
                    hit = lx0 <= bx + 7 && lx1 >= bx && ly0 <= by + 3 && ly1 >= by && s_zkey[jl] <= wzmax;
                }
                uint32_t todo = __ballot_sync(0xffffffffu, hit);
                if (!todo)
                    continue;
                while (todo)
                {
                    const uint32_t j = g + (uint32_t)(__ffs(todo) - 1);
                    todo &= todo - 1u;
                    const StagedTri& s = st[j];
                    const uint32_t fl = s.flags;
                    const int lx0 = fl & 31, lx1 = (fl >> 5) & 31, ly0 = (fl >> 10) & 31, ly1 = (fl >> 15) & 31;
                    if (lx < lx0 || lx > lx1 || ly < ly0 || ly > ly1)
                        continue;
                    uint64_t key;
                    if (fragment_key(s, lx, ly, less, key) && key < best)
                        best = key;
                }
                wzmax = __reduce_max_sync(0xffffffffu, (uint32_t)(best >> 32));
            }
            __syncthreads();
        }

        // both paths merged; the rank of the winner for k_shade
        if (SmallPath)
        {
            const uint64_t sk = s_key[pix];
            s_key[pix] = ~0ull;  // ready for the next tile (its first barrier orders this)
            if (sk < best)
                best = sk;
        }
        const uint32_t low = (uint32_t)best;
        const uint32_t rank = less ? low : ~low;
        const int px = (tileX << 4) + lx, py = (tileY << 4) + ly;
        if (px < f.width && py < f.height)
            a.tri_id[f.pix_base + (uint64_t)py * (uint32_t)f.width + (uint32_t)px] = rank;
    }
}

// Deferred shading of the winners (Renderer.cpp:272-350 shades every
// fragment and keeps the last; only the winner is shaded here): one thread
// per pixel finds the winner's raster triangle from its rank, recomputes its
// barycentrics and depth exactly (RasterTriangle.h:324-337), interpolates and
// shades, and writes colour, depth and the input-triangle id once.
__global__ void __launch_bounds__(256) k_shade(PassArgs a)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.total_pixels)
        return;
    const uint32_t rank = a.tri_id[i];
    const uint32_t nr = min(*(volatile uint32_t*)&a.counters[0], a.rtri_capacity);
    uint32_t ri = kNoTriangle;
    if (rank != 0)
    {
        // rank - 1 = flattened input triangle * 16 + fan index
        const uint32_t gi = (rank - 1u) >> 4, fan = (rank - 1u) & 15u;
        ri = gi < a.total_tris ? a.tri_first[gi] : kNoTriangle;
        // a clipped triangle's fan pieces are contiguous, in fan order
        for (int s = 0; s < kMaxPolygon && ri < nr && (a.rtris[ri].order & 15u) != fan; s++)
            ri++;
        if (ri >= nr || (a.rtris[ri].order & 15u) != fan)
            ri = kNoTriangle;
    }
    if (ri == kNoTriangle)
    {
        a.color[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        a.depth[i] = 1.0f;
        a.tri_id[i] = kNoTriangle;
        return;
    }
    const RTri t = a.rtris[ri];
    const FrameDesc& f = a.frames[t.meta >> 12];
    const uint64_t local = i - f.pix_base;
    const int px = (int)(local % (uint32_t)f.width), py = (int)(local / (uint32_t)f.width);
    const Edges e = tri_edges(t);
    const int cx = (px << 4) + 8, cy = (py << 4) + 8;
    const int n1 = wadd(wmul(e.B[1], wsub(cx, t.v2x)), wmul(e.C[1], wsub(cy, t.v2y)));
    const int n2 = wadd(wmul(e.B[2], wsub(cx, t.v2x)), wmul(e.C[2], wsub(cy, t.v2y)));
    const float L0 = fmul(__int2float_rn(n1), t.invDet);
    const float L1 = fmul(__int2float_rn(n2), t.invDet);
    const float L2 = fsub(fsub(1.0f, L0), L1);
    const float d = fadd(fadd(fmul(L0, t.z0), fmul(L1, t.z1)), fmul(L2, t.z2));
    const float3 c = shade_fragment(f, t, a.polys, L0, L1);
    a.color[i] = make_float4(c.x, c.y, c.z, 1.0f);
    a.depth[i] = d;
    a.tri_id[i] = t.order >> 4;
}

// -------------------------------------------------------------------------
// Renderer::GetBackBuffer compatibility: RGBA8, bottom-up (FrameBuffer.cpp:41).
__global__ void k_back_buffer(const float4* color, uchar4* out, int width, int height)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= width * height)
        return;
    const int x = i % width, y = i / width;
    const float4 c = color[i];
    auto b = [](float v) -> unsigned char {
        v = fminf(fmaxf(v, 0.0f), 1.0f);
        return (unsigned char)(v * 255.0f + 0.5f);
    };
    const bool covered = c.w > 0.0f;
    out[(size_t)(height - 1 - y) * width + x] = make_uchar4(b(c.x), b(c.y), b(c.z), covered ? 255 : 0);
}

// -------------------------------------------------------------------------


// Raster variants: 0 and 1 carry the triangle-parallel path (no register cap /
// capped for 5 blocks per SM); 2 is pixel-parallel only, capped for 6.
static int raster_occupancy(int variant)
{
    static int per_sm[3] = { 0, 0, 0 };
    if (!per_sm[variant])
    {
        cudaError_t e;
        if (variant == 0)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[0], k_raster<4, true>, kRasterThreads, 0);
        else if (variant == 1)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[1], k_raster<5, true>, kRasterThreads, 0);
        else
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[2], k_raster<6, false>, kRasterThreads, 0);
        if (e != cudaSuccess || per_sm[variant] < 1)
            per_sm[variant] = 1;
    }
    return per_sm[variant];
}

static int raster_blocks(int sms, const Tuning& t)
{
    const int variant = (t.raster_variant >= 0 && t.raster_variant <= 2) ? t.raster_variant : 1;
    int per = raster_occupancy(variant);
    if (t.raster_blocks_per_sm > 0 && t.raster_blocks_per_sm < per)
        per = t.raster_blocks_per_sm;
    return sms * per;
}

void prepare_kernels()
{
    raster_occupancy(0);
    raster_occupancy(1);
    raster_occupancy(2);
}

Tuning default_tuning()
{
    Tuning t;
    t.small_region = 32;
    t.raster_variant = 1;
    t.bin_blocks_per_sm = 8;
    t.raster_blocks_per_sm = 0;
    return t;
}

cudaError_t launch_pipeline(const PassArgs& a, cudaStream_t s, cudaEvent_t* ev)
{
    const int sms = a.num_sms > 0 ? a.num_sms : 148;
    const uint32_t nscan = (a.total_tiles + kScanBlock - 1) / kScanBlock;
    uint32_t* block_sums = a.tile_cursor + a.total_tiles + 1;  // scratch after the cursors
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(ev[i], s);
    };
    mark(0);
    k_clear<<<(a.total_tiles + 1 + 255) / 256 + 1, 256, 0, s>>>(a);
    if (a.total_vertices)
        k_vertex<<<(a.total_vertices + 255) / 256, 256, 0, s>>>(a);
    mark(1);
    if (a.total_tris)
    {
        k_setup<<<(a.total_tris + 255) / 256, 256, 0, s>>>(a);
        k_clip<<<sms * 4, 128, 0, s>>>(a);
    }
    mark(2);
    const int bin_blocks = sms * (a.tune.bin_blocks_per_sm > 0 ? a.tune.bin_blocks_per_sm : 8);
    k_bin<0><<<bin_blocks, 256, 0, s>>>(a);
    k_bin_big<<<sms * 4, 256, 0, s>>>(a);
    mark(3);
    k_scan_blocks<<<nscan, kScanThreads, 0, s>>>(a, block_sums);
    k_scan_spine<<<1, 1024, 0, s>>>(block_sums, nscan);
    k_scan_add<<<(a.total_tiles + 255) / 256 + 1, 256, 0, s>>>(a, block_sums, nscan);
    mark(4);
    k_bin<1><<<bin_blocks, 256, 0, s>>>(a);
    k_bin_move<<<sms * 4, 256, 0, s>>>(a);
    mark(5);
    if (a.tune.raster_variant == 2)
        k_raster<6, false><<<raster_blocks(sms, a.tune), kRasterThreads, 0, s>>>(a);
    else if (a.tune.raster_variant == 1)
        k_raster<5, true><<<raster_blocks(sms, a.tune), kRasterThreads, 0, s>>>(a);
    else
        k_raster<4, true><<<raster_blocks(sms, a.tune), kRasterThreads, 0, s>>>(a);
    mark(6);
    if (a.total_pixels)
        k_shade<<<(unsigned)((a.total_pixels + 255) / 256), 256, 0, s>>>(a);
    mark(7);
    return cudaGetLastError();
}

int kernels_per_pass(const PassArgs& a)
{
    return 9 + (a.total_vertices ? 1 : 0) + (a.total_tris ? 2 : 0) + (a.total_pixels ? 1 : 0);
}

cudaError_t launch_back_buffer(const float4* color, uint8_t* rgba8, int width, int height, cudaStream_t s)
{
    const int n = width * height;
    k_back_buffer<<<(n + 255) / 256, 256, 0, s>>>(color, reinterpret_cast<uchar4*>(rgba8), width, height);
    return cudaGetLastError();
}

}  // namespace edxr
