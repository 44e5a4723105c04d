// CUDA kernels of the EDXRaster GB300 pipeline (sm_103a).
//
// One pass renders any number of frames (a frame = one mesh seen by one
// camera); the plain path is a pass of one frame.  Stages:
//   k_clear        zero the per-tile counters and work queues;  Renderer.cpp:120-127
//                  the vertex stage of shared-vertex meshes
//   k_setup        clip = MVP * (p, 1), clip codes, fixed-point Shader.h:40-49,
//   k_clip         setup and the post-pass per input triangle;  Clipper.h:71-189,
//                  clipping of those that straddle a plane;     RasterTriangle.h:27-153
//                  the count pass of the binning
//   k_bin_*, scan  (triangle, 16x16 tile) decisions, counted,   Renderer.cpp:161-229
//                  scanned and scattered into per-tile bins
//   k_raster       persistent work items of tiles: coverage,   Renderer.cpp:248-350,
//                  depth test and winner per pixel, then the    Rasterizer.h:32-415,
//                  winner shaded: one write of colour, depth    FrameBuffer.cpp:54-68
//                  and triangle id per pixel
#include <cuda_runtime.h>

#include "edxr_device.cuh"

namespace edxr {

constexpr int kRasterThreads = 256;    // 8 warps, each on its own work items
constexpr uint32_t kBigChunk = 128;    // unsorted-list slots a k_bin_big warp reserves at a time
constexpr uint32_t kEmptySlot = 0xFFFFFFFFu;
constexpr uint32_t kSplitTile = 0x80000000u;  // item tag: the tile has several items (tiles < 2^24)

// Clip-space position of vertex v: clip = MVP * (p, 1) (DefaultVertexShader,
// Shader.h:40-49).
__device__ __forceinline__ float4 clip_position(const FrameDesc& f, uint32_t v)
{
    const float* p = reinterpret_cast<const float*>(f.positions + (size_t)v * f.pos_stride);
    return xform_point4(f.mvp, __ldg(p), __ldg(p + 1), __ldg(p + 2));
}

// Setup record of a vertex (vertex stage, for meshes whose vertices are
// shared by several triangles): inside the view volume (clip code 0) the
// projected vertex (x, y on the subpixel grid, z / w, 1 / w); otherwise
// (kVtxOutside, clip code).
constexpr int kVtxOutside = (int)0x80000000;

__device__ __forceinline__ int4 vertex_record(const FrameDesc& f, uint32_t v)
{
    const float4 c = clip_position(f, v);
    const uint32_t code = clip_code(c);
    if (code)
        return make_int4(kVtxOutside, (int)code, 0, 0);
    int vx, vy;
    float z, iw;
    project_vertex(f, c, vx, vy, z, iw);
    return make_int4(vx, vy, __float_as_int(z), __float_as_int(iw));
}

// -------------------------------------------------------------------------
// Clear of the per-tile counters and work queues, and the vertex stage.
__global__ void k_clear(PassArgs a)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    if (a.vrecs)
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.total_vertices; i += stride)
        {
            const uint32_t fi = find_frame(a.frames, a.num_frames, i, [](const FrameDesc& f) { return f.vtx_base; });
            const FrameDesc& f = a.frames[fi];
            a.vrecs[i] = vertex_record(f, i - f.vtx_base);
        }
    // several frames: the frame of every 256th triangle, where setup's
    // frame lookup starts (instead of a search over every frame)
    if (a.frame_of_block)
        for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b <= (a.total_tris >> 8); b += stride)
            a.frame_of_block[b] =
                find_frame(a.frames, a.num_frames, b << 8, [](const FrameDesc& f) { return f.tri_base; });
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= a.total_tiles; i += stride)
    {
        a.tile_count[i] = 0;
        a.tile_zocc[i] = 0xFFFFFFFFu;
        a.tile_cursor[i] = 0;
    }
    if (blockIdx.x == 0)
        for (int i = (int)threadIdx.x; i < kCounters; i += (int)blockDim.x)
            a.counters[i] = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < scan_blocks(a.total_tiles); i += stride)
        a.scan_status[i] = 0ull;
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        a.status->overflow = 0;
        a.status->error = 0;
        a.status->bins_needed = 0;
        a.status->raster_tris = 0;
        a.status->clipped_polys = 0;
        a.status->big_tris = 0;
        a.status->bin_entries = 0;
    }
}

// -------------------------------------------------------------------------
// -------------------------------------------------------------------------
// Binning.  Every non-rejected (triangle, tile) pair is counted in its tile
// and kept as (tile, raster triangle << 2 | decision) in an unsorted list;
// after the scan of the counts, k_bin_move moves the entries into their
// bins.  Triangles the reference treats as small are binned by the thread
// that sets them up (k_setup, k_clip); the others by one warp each with the
// full decision of quad_decisions (k_bin_big).
//
// bin_count_tile counts one entry of `tile`.  Neighbouring triangles of a
// warp often land in the same tile: lanes with equal tiles share one atomic,
// issued by the lowest lane.
__device__ __forceinline__ void bin_count_tile(const PassArgs& a, uint32_t tile)
{
    const uint32_t act = __activemask();
    const uint32_t peers = __match_any_sync(act, tile);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1)
        atomicAdd(&a.tile_count[tile], (uint32_t)__popc(peers));
}

// A small triangle's entries.  The reference rasterizes a small triangle
// with FineRasterize in every tile of its range (Renderer.cpp:173-180), so
// the decision is "fine" where the quad-aligned bounding box meets the
// screen.  Tiles where no pixel centre can be covered get no entry.
struct SmallTiles
{
    int tx0, tx1, ty0, ty1;
};

// The tile range of a small triangle's entries and their number.
__device__ __forceinline__ uint32_t small_tiles(const PassArgs& a, const FrameDesc& f, const RTri& t, const BinGeom& g,
                                               SmallTiles& st)
{
    // Without wraparound only points inside the vertices' bounding box can be
    // covered: with one sample per pixel the pixels whose centre is in it,
    // with several (each inside its own pixel) the pixels the box overlaps.
    // Otherwise the reference's quad-aligned region.
    const bool wfree = wrap_free(t);
    const bool tight = a.msaa_log2 == 0 && wfree, box = a.msaa_log2 != 0 && wfree;
    const int x0 = max(tight ? g.cx0 : box ? g.bbx0 : g.bbx0 & ~1, 0);
    const int x1 = min(tight ? g.cx1 : box ? g.bbx1 : g.bbx1 | 1, f.width - 1);
    const int y0 = max(tight ? g.cy0 : box ? g.bby0 : g.bby0 & ~1, 0);
    const int y1 = min(tight ? g.cy1 : box ? g.bby1 : g.bby1 | 1, f.height - 1);
    if (x0 > x1 || y0 > y1)
        return 0;
    st.tx0 = x0 >> kTileLog2;
    st.tx1 = x1 >> kTileLog2;
    st.ty0 = y0 >> kTileLog2;
    st.ty1 = y1 >> kTileLog2;
    return (uint32_t)((st.tx1 - st.tx0 + 1) * (st.ty1 - st.ty0 + 1));
}

// Counts a small triangle's entries in their tiles and keeps them in the
// unsorted list from `slot` on, up to its stripe's end (the caller reserved
// their number; entries past the end are dropped, the frame overflows).
__device__ __forceinline__ void bin_small(const PassArgs& a, const FrameDesc& f, uint32_t ri, const SmallTiles& st,
                                          uint64_t slot, uint64_t end)
{
    for (int ty = st.ty0; ty <= st.ty1; ty++)
        for (int tx = st.tx0; tx <= st.tx1; tx++)
        {
            const uint32_t tile = f.tile_base + (uint32_t)(ty * f.tdx + tx);
            bin_count_tile(a, tile);
            if (slot < end)
                a.bin_tmp[slot] = make_uint2(tile, (ri << 2) | kDecisionFine);
            slot++;
        }
}

// Lower bound (as a depth key) of every depth the reference computes for the
// triangle at a pixel it rasterizes, or 0 (never culled) when the triangle is
// large enough for int32 edge values to wrap.  Without wraparound the
// barycentrics of rasterized pixels are within a few ulps of [0, 1], so the
// computed depth is at least min(z) minus a few ulps of the |z| sum.
__device__ __forceinline__ uint32_t zmin_key(const RTri& t, bool wf)
{
    if (!wf)
        return 0u;
    const float zmin = fminf(t.z0, fminf(t.z1, t.z2));
    const float margin = 2e-6f * (fabsf(t.z0) + fabsf(t.z1) + fabsf(t.z2)) + 1e-30f;
    const float lo = zmin - margin;
    return (lo == lo) ? depth_key(lo) : 0u;
}

// Stripe of the unsorted bin list a warp appends to, its fill counter and
// its first slot.
__device__ __forceinline__ uint32_t warp_stripe()
{
    return ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) % (uint32_t)kBinStripes;
}
__device__ __forceinline__ uint32_t* stripe_counter(const PassArgs& a, uint32_t r)
{
    return a.counters + kStripeBase + r * kStripeStride;
}
__device__ __forceinline__ uint64_t stripe_begin(const PassArgs& a, uint32_t r)
{
    return (uint64_t)r * stripe_slots(a.bin_capacity);
}

// A big triangle (bounding box over more than 2x2 reference tiles) goes to
// the list k_bin_big bins warp-cooperatively, appended to with one atomic
// per warp.
__device__ __forceinline__ void bin_big_append(const PassArgs& a, uint32_t ri, bool big)
{
    const uint32_t act = __activemask();
    const uint32_t bigs = __ballot_sync(act, big);
    if (!big)
        return;
    const uint32_t lane = threadIdx.x & 31;
    const int leader = __ffs(bigs) - 1;
    uint32_t b = 0;
    if ((int)lane == leader)
        b = atomicAdd(&a.counters[2], (uint32_t)__popc(bigs));
    b = __shfl_sync(bigs, b, leader) + (uint32_t)__popc(bigs & ((1u << lane) - 1u));
    if (b < a.big_capacity)
        a.big_list[b] = ri;
}


// Appends n slots for this lane with one atomic per warp on `counter`;
// returns the lane's first slot.  Every lane of the warp must call it.
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

// Frame of flattened input triangle gi: from its 256-block's frame, forward
// over the frames that start at or before it (find_frame's answer: the last
// frame whose first triangle is at or before gi).
__device__ __forceinline__ uint32_t frame_of_triangle(const PassArgs& a, uint32_t gi)
{
    if (!a.frame_of_block)
        return find_frame(a.frames, a.num_frames, gi, [](const FrameDesc& f) { return f.tri_base; });
    uint32_t fi = a.frame_of_block[gi >> 8];
    while (fi + 1 < a.num_frames && a.frames[fi + 1].tri_base <= gi)
        fi++;
    return fi;
}

// Setup of the triangles that need no clipping (all clip codes zero), one
// thread per input triangle; triangles that straddle a clip plane are queued
// for k_clip, triangles outside one plane are dropped (Clipper.h:103-109).
// A small set-up triangle is binned here as well.  A set-up triangle's
// record goes to its own slot (no append); the clip queue and the warp's
// stripe of the unsorted bin list take one atomic per warp each.
__global__ void __launch_bounds__(256, 6) k_setup(PassArgs a)
{
    const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31;
    uint32_t fi = 0, tri = 0;
    int nOut = 0;
    bool straddle = false, big = false;
    uint32_t nent = 0;
    SmallTiles st;
    RTri t;
    if (gi < a.total_tris)
    {
        fi = frame_of_triangle(a, gi);
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
            uint32_t k0, k1, k2;
            if (a.vrecs)
            {
                // projected by the vertex stage
                const int4 r0 = a.vrecs[f.vtx_base + i0], r1 = a.vrecs[f.vtx_base + i1], r2 = a.vrecs[f.vtx_base + i2];
                k0 = r0.x == kVtxOutside ? (uint32_t)r0.y : 0u;
                k1 = r1.x == kVtxOutside ? (uint32_t)r1.y : 0u;
                k2 = r2.x == kVtxOutside ? (uint32_t)r2.y : 0u;
                if ((k0 | k1 | k2) == 0)
                {
                    const int vx[3] = { r0.x, r1.x, r2.x }, vy[3] = { r0.y, r1.y, r2.y };
                    const float zp[3] = { __int_as_float(r0.z), __int_as_float(r1.z), __int_as_float(r2.z) };
                    const float iw[3] = { __int_as_float(r0.w), __int_as_float(r1.w), __int_as_float(r2.w) };
                    nOut = setup_projected(vx, vy, zp, iw, t) ? 1 : 0;
                }
            }
            else
            {
                const float4 c0 = clip_position(f, i0);
                const float4 c1 = clip_position(f, i1);
                const float4 c2 = clip_position(f, i2);
                k0 = clip_code(c0);
                k1 = clip_code(c1);
                k2 = clip_code(c2);
                if ((k0 | k1 | k2) == 0)
                    nOut = setup_triangle(f, c0, c1, c2, t) ? 1 : 0;
            }
            if (nOut)
            {
                const BinGeom g = bin_geom(t, f);
                big = !g.small;
                if (g.small)
                    nent = small_tiles(a, f, t, g, st);
            }
            straddle = (k0 | k1 | k2) != 0 && !(k0 & k1 & k2);
        }
    }
    // warp-wide exclusive scans of the queued triangles and of the bin
    // entries; one atomic per warp on the clip queue (few warps have any)
    // and on the warp's stripe of the unsorted list
    uint32_t qincl = straddle ? 1u : 0u, eincl = nent;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t v = __shfl_up_sync(0xffffffffu, qincl, o);
        const uint32_t ve = __shfl_up_sync(0xffffffffu, eincl, o);
        if (lane >= (uint32_t)o)
        {
            qincl += v;
            eincl += ve;
        }
    }
    const uint32_t stripe = warp_stripe();
    const uint32_t survivors = __popc(__ballot_sync(0xffffffffu, nOut != 0));
    uint32_t qbase = 0, ebase = 0;
    if (lane == 31)
    {
        if (survivors)
            atomicAdd(stripe_counter(a, stripe) + 1, survivors);  // statistics
        qbase = qincl ? atomicAdd(&a.counters[4], qincl) : 0u;
        ebase = eincl ? atomicAdd(stripe_counter(a, stripe), eincl) : 0u;
    }
    qbase = __shfl_sync(0xffffffffu, qbase, 31);
    ebase = __shfl_sync(0xffffffffu, ebase, 31);
    if (straddle)
    {
        const uint32_t q = qbase + qincl - 1u;
        if (q < a.poly_capacity)
            a.clip_list[q] = gi;
    }
    // an unclipped triangle's record sits at its flattened index
    const uint64_t sbegin = stripe_begin(a, stripe);
    const uint64_t slot = sbegin + ebase + eincl - nent;
    if (nOut)
    {
        t.order = tri << 4;
        t.meta |= fi << 12;
        t.poly = kUnclipped;
        a.rtris[gi] = t;
        a.rtri_zlo[gi] = zmin_key(t, wrap_free(t));
    }
    bin_big_append(a, gi, nOut && big);
    if (nOut && nent)
        bin_small(a, a.frames[fi], gi, st, slot, sbegin + stripe_slots(a.bin_capacity));
}

// Clipping of the queued triangles (Clipper.h:107-171): Sutherland-Hodgman,
// fan triangulation, setup of each fan triangle.  Each clipped triangle
// reserves n - 2 consecutive raster-triangle slots, fan piece k - 1 (fan
// vertices 0, k - 1, k) in slot first + k - 2; a piece that setup culls
// leaves its slot unused.  Its polygon record is the one of its queue
// position.  Two ways to spread the work over the lanes, chosen by the
// queue length (the kernel is latency-bound either way):
//  - short queues (one round of the grid's 16-lane groups): a group clips
//    one triangle with one polygon vertex per lane (a polygon has at most
//    kMaxPolygon = 16 vertices), so the polygon stays in registers: per
//    plane each lane classifies its edge (its vertex and the next), emits 0,
//    1 or 2 vertices, and a scan over the group places them in the order of
//    the serial loop (Clipper::ClipPolygon, Clipper.h:235-288);
//  - long queues: the first `per` lanes of a warp (per <= kClipPer) clip one
//    triangle each with the serial loop, and the warp's fan pieces are then
//    set up one per lane.
constexpr int kClipThreads = 128;
constexpr int kClipWarps = kClipThreads / 32;
constexpr int kClipLanes = 16;
constexpr int kClipPer = 8;
static_assert(kClipLanes == kMaxPolygon, "one lane per polygon vertex");

// Bit of plane k in the order L, R, B, T, F, N.
__device__ __forceinline__ uint32_t plane_bit(int k)
{
    return k < 4 ? 1u << k : (k == 4 ? (uint32_t)kFar : (uint32_t)kNear);
}

// Clipper::ClipPolygon (Clipper.h:235-288), one lane: Sutherland-Hodgman
// against the planes in planeCode, in the order L, R, B, T, F, N, then the
// polygon is dropped when any vertex has w <= 0.  The polygon starts in buf0
// and alternates between buf0 and buf1; returns the vertex count and sets
// res to the buffer that holds the result.
__device__ __forceinline__ int clip_polygon(PolyVert* buf0, PolyVert* buf1, uint32_t planeCode, PolyVert*& res)
{
    PolyVert* src = buf0;
    PolyVert* dst = buf1;
    int n = 3;
#pragma unroll 1
    for (int k = 0; k < 6; k++)
    {
        if (!(planeCode & plane_bit(k)))
            continue;
        int m = 0;
        // edges (i, i + 1) from i = 0, the first vertex carried in registers
        PolyVert v0 = src[0];
        bool in0 = plane_inside(k, v0.p);
        for (int i = 0; i < n; i++)
        {
            const PolyVert v1 = src[(i + 1 == n) ? 0 : i + 1];
            const bool in1 = plane_inside(k, v1.p);
            if (in0)
            {
                if (m < kMaxPolygon) dst[m++] = in1 ? v1 : plane_cut(k, v0, v1);
            }
            else if (in1)
            {
                if (m < kMaxPolygon) dst[m++] = plane_cut(k, v0, v1);
                if (m < kMaxPolygon) dst[m++] = v1;
            }
            v0 = v1;
            in0 = in1;
        }
        PolyVert* t = src;
        src = dst;
        dst = t;
        n = m;
    }
    res = src;
    for (int i = 0; i < n; i++)
        if (src[i].p.w <= 0.0f)
            return 0;
    return n;
}

// Clipper.h:121-152: a polygon vertex whose weight is exactly one on a source
// vertex is that source vertex (position and attributes); the others are
// new.  Returns the source index, or -1, and makes the weights exact.
__device__ __forceinline__ int source_vertex(PolyVert& v)
{
    int sv = -1;
    if (v.w0 == 1.0f) sv = 0;
    else if (v.w1 == 1.0f) sv = 1;
    else if (v.w2 == 1.0f) sv = 2;
    if (sv >= 0)
    {
        v.w0 = (sv == 0) ? 1.f : 0.f;
        v.w1 = (sv == 1) ? 1.f : 0.f;
        v.w2 = (sv == 2) ? 1.f : 0.f;
    }
    return sv;
}

// Slots of a warp's fan pieces and the capacity checks: `pieces` is this
// lane's count (0 for lanes that hold no triangle); returns its first slot
// and clears `pieces` when a capacity is exceeded.
__device__ __forceinline__ uint32_t reserve_pieces(const PassArgs& a, int& pieces, uint32_t q)
{
    const uint32_t first = a.total_tris + warp_append(&a.counters[0], pieces);
    if (pieces && (uint64_t)first + (uint32_t)pieces > a.rtri_capacity)
    {
        atomicOr(&a.status->overflow, 2u);
        pieces = 0;
    }
    if (pieces && q >= a.poly_capacity)
    {
        atomicOr(&a.status->overflow, 4u);
        pieces = 0;
    }
    return first;
}

// Setup and binning of one fan piece (c0, c1, c2 in clip space): piece `fan`
// of input triangle `tri` of frame fi, clipped polygon `poly`, slot ri.
// Every lane of the warp calls it; lanes with has == false hold no piece.
__device__ __forceinline__ void clip_piece(const PassArgs& a, bool has, uint32_t fi, uint32_t tri, uint32_t poly,
                                           uint32_t fan, uint32_t ri, float4 c0, float4 c1, float4 c2)
{
    const FrameDesc& f = a.frames[fi];
    bool big = false, kept = false;
    uint32_t nent = 0;
    SmallTiles st;
    RTri tk;
    if (has && setup_triangle(f, c0, c1, c2, tk))
    {
        tk.order = (tri << 4) | fan;
        tk.meta |= fi << 12;
        tk.poly = (poly << 4) | (fan + 1u);
        kept = true;
        a.rtris[ri] = tk;
        a.rtri_zlo[ri] = zmin_key(tk, wrap_free(tk));
        const BinGeom bg = bin_geom(tk, f);
        big = !bg.small;
        if (bg.small)
            nent = small_tiles(a, f, tk, bg, st);
    }
    const uint32_t kept_lanes = __ballot_sync(0xffffffffu, kept);
    if ((threadIdx.x & 31) == 0 && kept_lanes)
        atomicAdd(&a.counters[11], (uint32_t)__popc(kept_lanes));
    bin_big_append(a, ri, big);
    const uint32_t stripe = warp_stripe();
    const uint64_t sbegin = stripe_begin(a, stripe);
    const uint64_t slot = sbegin + warp_append(stripe_counter(a, stripe), (int)nent);
    if (nent)
        bin_small(a, f, ri, st, slot, sbegin + stripe_slots(a.bin_capacity));
}

// Vertex of lane `src` (within the 16-lane group) of every lane's group.
__device__ __forceinline__ PolyVert shfl_vert(const PolyVert& v, int src)
{
    PolyVert r;
    r.p.x = __shfl_sync(0xffffffffu, v.p.x, src, kClipLanes);
    r.p.y = __shfl_sync(0xffffffffu, v.p.y, src, kClipLanes);
    r.p.z = __shfl_sync(0xffffffffu, v.p.z, src, kClipLanes);
    r.p.w = __shfl_sync(0xffffffffu, v.p.w, src, kClipLanes);
    r.w0 = __shfl_sync(0xffffffffu, v.w0, src, kClipLanes);
    r.w1 = __shfl_sync(0xffffffffu, v.w1, src, kClipLanes);
    r.w2 = __shfl_sync(0xffffffffu, v.w2, src, kClipLanes);
    return r;
}
__device__ __forceinline__ float4 shfl_f4(float4 v, int src)
{
    return make_float4(__shfl_sync(0xffffffffu, v.x, src, kClipLanes), __shfl_sync(0xffffffffu, v.y, src, kClipLanes),
                       __shfl_sync(0xffffffffu, v.z, src, kClipLanes), __shfl_sync(0xffffffffu, v.w, src, kClipLanes));
}

// Short queues: one 16-lane group per triangle, q < nq <= the grid's groups.
__device__ __forceinline__ void clip_groups(const PassArgs& a, uint32_t nq)
{
    const uint32_t lane = threadIdx.x & 31;
    const int g = (int)(lane & 15u);  // vertex lane within the group
    const uint32_t gmask = 0xFFFFu << (lane & 16u);
    const uint32_t q = (blockIdx.x * kClipThreads + threadIdx.x) / kClipLanes;
    uint32_t gi = 0, fi = 0, tri = 0, code = 0;
    PolyVert v = { make_float4(0.f, 0.f, 0.f, 0.f), 0.f, 0.f, 0.f };
    int n = 0;
    if (q < nq)
    {
        gi = a.clip_list[q];
        fi = frame_of_triangle(a, gi);
        const FrameDesc& f = a.frames[fi];
        tri = gi - f.tri_base;
        n = 3;
        if (g < 3)
        {
            v.p = clip_position(f, __ldg(f.indices + 3 * (size_t)tri + g));
            v.w0 = g == 0 ? 1.f : 0.f;
            v.w1 = g == 1 ? 1.f : 0.f;
            v.w2 = g == 2 ? 1.f : 0.f;
            code = clip_code(v.p);
        }
    }
    const float4 src = v.p;  // source vertex g (g < 3)
    const uint32_t k0 = __shfl_sync(0xffffffffu, code, 0, kClipLanes);
    const uint32_t k1 = __shfl_sync(0xffffffffu, code, 1, kClipLanes);
    const uint32_t k2 = __shfl_sync(0xffffffffu, code, 2, kClipLanes);
    const uint32_t planes = (k0 ^ k1) | (k1 ^ k2) | (k2 ^ k0);
    const uint32_t any = __reduce_or_sync(0xffffffffu, planes);
#pragma unroll 1
    for (int k = 0; k < 6; k++)
    {
        const uint32_t bit = plane_bit(k);
        if (!(any & bit))
            continue;
        // edge (g, g + 1 mod n): its end vertex, the cut, the emissions
        const PolyVert v1 = shfl_vert(v, (g + 1 >= n) ? 0 : g + 1);
        const bool valid = g < n;
        const bool in0 = valid && plane_inside(k, v.p);
        const bool in1 = valid && plane_inside(k, v1.p);
        const int c = !valid ? 0 : (in0 ? 1 : (in1 ? 2 : 0));
        PolyVert e0 = v1;
        if (valid && in0 != in1)
            e0 = plane_cut(k, v, v1);
        int incl = c;
#pragma unroll
        for (int o = 1; o < kClipLanes; o <<= 1)
        {
            const int t = __shfl_up_sync(0xffffffffu, incl, o, kClipLanes);
            if (g >= o) incl += t;
        }
        const int m = min(__shfl_sync(0xffffffffu, incl, kClipLanes - 1, kClipLanes), kMaxPolygon);
        // output vertex g: emission g - excl(s) of the first lane s whose
        // inclusive count exceeds g
        int s = 0;
#pragma unroll
        for (int st = kClipLanes / 2; st >= 1; st >>= 1)
        {
            const int t = __shfl_sync(0xffffffffu, incl, s + st - 1, kClipLanes);
            if (t <= g) s += st;
        }
        const int which = g - __shfl_sync(0xffffffffu, incl - c, s, kClipLanes);
        const PolyVert first = shfl_vert(e0, s);
        const PolyVert second = shfl_vert(v1, s);
        if (planes & bit)
        {
            if (g < m)
                v = which == 0 ? first : second;
            n = m;
        }
    }
    // the polygon is dropped when any vertex has w <= 0
    if (__ballot_sync(0xffffffffu, g < n && v.p.w <= 0.0f) & gmask)
        n = 0;
    const int sv = source_vertex(v);
    const float4 sp = shfl_f4(src, sv < 0 ? 0 : sv);
    if (sv >= 0)
        v.p = sp;
    int pieces = (g == 0 && n >= 3) ? n - 2 : 0;
    const uint32_t first = __shfl_sync(0xffffffffu, reserve_pieces(a, pieces, q), 0, kClipLanes);
    pieces = __shfl_sync(0xffffffffu, pieces, 0, kClipLanes);
    if (pieces)
    {
        ClipPoly& P = a.polys[q];
        if (g < n)
        {
            P.w[g][0] = v.w0;
            P.w[g][1] = v.w1;
            P.w[g][2] = v.w2;
        }
        if (g == 0)
        {
            P.n = (uint32_t)n;
            a.tri_first[gi] = first;
        }
    }
    // lane g: piece g + 1, fan vertices 0, g + 1, g + 2
    const float4 f0 = shfl_f4(v.p, 0);
    const float4 f1 = shfl_f4(v.p, min(g + 1, kClipLanes - 1));
    const float4 f2 = shfl_f4(v.p, min(g + 2, kClipLanes - 1));
    clip_piece(a, g < pieces, fi, tri, q, (uint32_t)g + 1u, first + (uint32_t)g, f0, f1, f2);
}

// Long queues: `per` triangles per warp and round, clipped by one lane each.
__device__ __forceinline__ void clip_lanes(const PassArgs& a, uint32_t nq, float4 (*s_vc)[kMaxPolygon])
{
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nwarps = gridDim.x * kClipWarps;
    uint32_t per = 1;
    while (per < (uint32_t)kClipPer && (uint64_t)per * nwarps < nq)
        per <<= 1;
    const uint64_t span = (uint64_t)per * nwarps;
    const uint32_t rounds = (uint32_t)((nq + span - 1) / span);
    for (uint32_t r = 0; r < rounds; r++)
    {
        const uint64_t q64 = ((uint64_t)r * nwarps + blockIdx.x * kClipWarps + warp) * per + lane;
        const uint32_t q = (uint32_t)min(q64, (uint64_t)0xFFFFFFFFu);
        PolyVert buf0[kMaxPolygon], buf1[kMaxPolygon];
        PolyVert* poly = buf0;
        int n = 0;
        uint32_t gi = 0, fi = 0, tri = 0;
        if (lane < per && q64 < nq)
        {
            gi = a.clip_list[q];
            fi = frame_of_triangle(a, gi);
            const FrameDesc& f = a.frames[fi];
            tri = gi - f.tri_base;
            const float4 c0 = clip_position(f, __ldg(f.indices + 3 * (size_t)tri));
            const float4 c1 = clip_position(f, __ldg(f.indices + 3 * (size_t)tri + 1));
            const float4 c2 = clip_position(f, __ldg(f.indices + 3 * (size_t)tri + 2));
            const uint32_t k0 = clip_code(c0), k1 = clip_code(c1), k2 = clip_code(c2);
            buf0[0] = { c0, 1.f, 0.f, 0.f };
            buf0[1] = { c1, 0.f, 1.f, 0.f };
            buf0[2] = { c2, 0.f, 0.f, 1.f };
            n = clip_polygon(buf0, buf1, (k0 ^ k1) | (k1 ^ k2) | (k2 ^ k0), poly);
            const float4 src[3] = { c0, c1, c2 };
            for (int j = 0; j < n; j++)
            {
                const int sv = source_vertex(poly[j]);
                s_vc[lane][j] = sv >= 0 ? src[sv] : poly[j].p;
            }
        }
        int pieces = n >= 3 ? n - 2 : 0;
        const uint32_t first = reserve_pieces(a, pieces, q);
        if (pieces)
        {
            ClipPoly& P = a.polys[q];
            for (int j = 0; j < n; j++)
            {
                P.w[j][0] = poly[j].w0;
                P.w[j][1] = poly[j].w1;
                P.w[j][2] = poly[j].w2;
            }
            P.n = (uint32_t)n;
            a.tri_first[gi] = first;
        }
        // the warp's pieces, numbered across its lanes and taken 32 at a time
        int incl = pieces;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        __syncwarp();
        for (int base = 0; base < total; base += 32)
        {
            const int p = base + (int)lane;
            // owner: the first lane whose inclusive count exceeds p
            int j = 0;
#pragma unroll
            for (int st = 16; st >= 1; st >>= 1)
            {
                const int v = __shfl_sync(0xffffffffu, incl, j + st - 1);
                if (v <= p) j += st;
            }
            const int k = p - __shfl_sync(0xffffffffu, incl - pieces, j) + 2;
            const uint32_t jfirst = __shfl_sync(0xffffffffu, first, j);
            const uint32_t jfi = __shfl_sync(0xffffffffu, fi, j);
            const uint32_t jtri = __shfl_sync(0xffffffffu, tri, j);
            const uint32_t jq = __shfl_sync(0xffffffffu, q, j);
            const bool has = p < total;
            const float4* vj = s_vc[j & (kClipPer - 1)];
            float4 c0 = make_float4(0.f, 0.f, 0.f, 1.f), c1 = c0, c2 = c0;
            if (has)
            {
                c0 = vj[0];
                c1 = vj[k - 1];
                c2 = vj[k];
            }
            clip_piece(a, has, jfi, jtri, jq, (uint32_t)(k - 1), jfirst + (uint32_t)(k - 2), c0, c1, c2);
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(kClipThreads) k_clip(PassArgs a)
{
    __shared__ float4 s_vc[kClipWarps][kClipPer][kMaxPolygon];
    const uint32_t nq = min(*(volatile uint32_t*)&a.counters[4], a.poly_capacity);
    if (nq <= gridDim.x * (uint32_t)(kClipThreads / kClipLanes))
        clip_groups(a, nq);
    else
        clip_lanes(a, nq, s_vc[threadIdx.x >> 5]);
}

// Scatter of the unsorted entries into their bins (after the scan); empty
// slots and entries hidden behind their tile's occluder are skipped, so a
// bin holds its tile's first tile_cursor entries.
__global__ void __launch_bounds__(256) k_bin_move(PassArgs a)
{
    // the filled parts of the stripes (slots past a stripe's end were
    // dropped: overflow), numbered one after another
    __shared__ uint32_t s_first[kBinStripes + 1];
    // a pass that reported an error (a scan wait that ran out, a bad index)
    // fails as a whole: its offsets may be wrong, so nothing is scattered
    if (*(volatile uint32_t*)&a.status->error)
        return;
    const uint64_t R = stripe_slots(a.bin_capacity);
    const uint32_t lane = threadIdx.x & 31;
    if (threadIdx.x < 32)
    {
        static_assert(kBinStripes == 32, "one lane per stripe");
        const uint32_t m = (uint32_t)min((uint64_t)*(volatile uint32_t*)stripe_counter(a, lane), R);
        uint32_t incl = m;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += v;
        }
        s_first[lane] = incl - m;
        if (lane == 31)
            s_first[32] = incl;
    }
    __syncthreads();
    const uint32_t total = s_first[kBinStripes];
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (total + stride - 1) / stride;
    for (uint32_t rd = 0; rd < rounds; rd++)
    {
        const uint32_t j = rd * stride + blockIdx.x * blockDim.x + threadIdx.x;
        uint2 e = make_uint2(kEmptySlot, 0u);
        if (j < total)
        {
            // stripe of entry j: the last one starting at or before it
            uint32_t r = 0;
#pragma unroll
            for (uint32_t st = 16; st >= 1; st >>= 1)
                if (s_first[r + st] <= j) r += st;
            e = a.bin_tmp[(uint64_t)r * R + (j - s_first[r])];
            // an entry wholly behind its tile's occluder is dropped: the
            // raster's depth bound would skip it at staging (its nearest
            // depth beyond min(occluder bound, clear depth))
            if (e.x != kEmptySlot)
            {
                const uint32_t zocc = a.tile_zocc[e.x];
                const uint32_t ri = e.y >> 2;
                if (zocc != 0xFFFFFFFFu && ri < a.rtri_capacity && a.rtri_zlo[ri] > min(zocc, 0xBF800000u))
                    e.x = kEmptySlot;
            }
        }
        uint32_t base = 0;
        if (a.vrecs)
        {
            // a mesh with shared vertices: neighbouring lanes hold entries
            // of neighbouring triangles, interleaved over the same few
            // tiles; all lanes with equal tiles share one atomic
            const uint32_t peers = __match_any_sync(0xffffffffu, e.x);
            const int leader = __ffs(peers) - 1;
            if ((int)lane == leader && e.x != kEmptySlot)
                base = atomicAdd(&a.tile_cursor[e.x], (uint32_t)__popc(peers));
            base = __shfl_sync(0xffffffffu, base, leader) + (uint32_t)__popc(peers & ((1u << lane) - 1u));
        }
        else
        {
            // a triangle soup: lanes rarely share a tile, except in runs
            // of consecutive lanes, which share one atomic
            const uint32_t prev = __shfl_up_sync(0xffffffffu, e.x, 1);
            const uint32_t heads = __ballot_sync(0xffffffffu, lane == 0 || e.x != prev);
            const uint32_t upto = 0xffffffffu >> (31 - lane);  // lanes 0..lane
            const uint32_t head = 31 - __clz(heads & upto);
            if (lane == head && e.x != kEmptySlot)
            {
                const uint32_t later = heads & ~upto;
                const uint32_t end = later ? (uint32_t)__ffs(later) - 1u : 32u;
                base = atomicAdd(&a.tile_cursor[e.x], end - lane);
            }
            base = __shfl_sync(0xffffffffu, base, head) + (lane - head);
        }
        if (e.x == kEmptySlot)
            continue;
        const uint64_t pos = (uint64_t)a.tile_offset[e.x] + base;
        if (pos < a.bin_capacity)
            a.bins[pos] = e.y;
    }
}

// Upper bound (as a depth key) of every depth the reference computes for
// the triangle at a pixel of a 16x16 block it trivially accepts, or ~0 (no
// bound) when its edge values can wrap or its depths are not finite.  The
// block's corners are inside every edge, so are all its pixel centres: the
// barycentrics are within a few ulps of [0, 1] and the depth at most max(z)
// plus a few ulps of the |z| sum.  Every entry of the tile whose lower bound
// lies beyond it loses at every pixel to this triangle's fragment.
__device__ __forceinline__ uint32_t zmax_key(const RTri& t)
{
    if (!wrap_free(t))
        return 0xFFFFFFFFu;
    const float zmax = fmaxf(t.z0, fmaxf(t.z1, t.z2));
    const float margin = 2e-6f * (fabsf(t.z0) + fabsf(t.z1) + fabsf(t.z2)) + 1e-30f;
    const float hi = zmax + margin;
    return (hi == hi && fabsf(hi) <= 3.0e38f && fabsf(t.invDet) <= 3.0e38f) ? depth_key(hi) : 0xFFFFFFFFu;
}

// Big triangles, up to 32 at a time per warp: their (triangle, 32x32 reference
// tile) pairs are numbered across the warp and taken 32 at a time, each lane
// deciding the four quadrants of its pair's tile, so a triangle with few
// tiles does not leave lanes idle.  Each entry is counted in its tile and
// kept in the unsorted list, which the warp fills from slots it reserves
// kBigChunk at a time (one atomic on the shared counter per chunk); slots
// it leaves unused are marked empty.
__global__ void __launch_bounds__(256, 4) k_bin_big(PassArgs a)
{
    const uint32_t nb = min(*(volatile uint32_t*)&a.counters[2], a.big_capacity);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    // the warp's current chunk of its stripe of the unsorted list
    const uint32_t stripe = warp_stripe();
    const uint64_t send = stripe_begin(a, stripe) + stripe_slots(a.bin_capacity);
    uint64_t cbase = 0;
    uint32_t cleft = 0;
    auto mark_empty = [&]() {
        for (uint32_t k = lane; k < cleft; k += 32)
            if (cbase + k < send)
                a.bin_tmp[cbase + k] = make_uint2(kEmptySlot, 0u);
    };
    // batches of up to 32 triangles, small enough that every warp gets one
    const uint32_t batch = min(32u, max(1u, (nb + nw - 1) / nw));
    const bool early_cull = nb >= a.total_tiles;
    for (uint32_t b0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * batch; b0 < nb; b0 += nw * batch)
    {
        // this lane's triangle of the batch and its number of 32x32 tiles
        uint32_t mine = kNoTriangle, mine_zocc = 0xFFFFFFFFu;
        int n = 0;
        if (lane < batch && b0 + lane < nb)
        {
            mine = a.big_list[b0 + lane];
            const RTri t = a.rtris[mine];
            const BinGeom g = bin_geom(t, a.frames[t.meta >> 12]);
            n = (g.t32x1 - g.t32x0 + 1) * (g.t32y1 - g.t32y0 + 1);
            mine_zocc = zmax_key(t);
        }
        int incl = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += v;
        }
        const int pairs = __shfl_sync(0xffffffffu, incl, 31);
        for (int base = 0; base < pairs; base += 32)
        {
            const int p = base + (int)lane;
            // owner: the first lane whose inclusive count exceeds p
            int j = 0;
#pragma unroll
            for (int st = 16; st >= 1; st >>= 1)
            {
                const int v = __shfl_sync(0xffffffffu, incl, j + st - 1);
                if (v <= p) j += st;
            }
            const int first = __shfl_sync(0xffffffffu, incl - n, j);
            const uint32_t ri = __shfl_sync(0xffffffffu, mine, j);
            // an accepted quadrant is covered whole: the triangle's far depth
            // bounds the tile
            const uint32_t zocc = __shfl_sync(0xffffffffu, mine_zocc, j);
            uint32_t dq = 0, tile00 = 0;
            int tdx = 0;
            if (p < pairs)
            {
                const RTri t = a.rtris[ri];
                const FrameDesc& f = a.frames[t.meta >> 12];
                const BinGeom g = bin_geom(t, f);
                const Edges e = tri_edges(t);
                const int nx = g.t32x1 - g.t32x0 + 1, local = p - first;
                const int T32y = g.t32y0 + local / nx, T32x = g.t32x0 + local - (local / nx) * nx;
                dq = quad_decisions(t, e, g, f, T32x, T32y);
                tdx = f.tdx;
                tile00 = f.tile_base + (uint32_t)(2 * T32y * f.tdx + 2 * T32x);
                // a quadrant already hidden behind its tile's occluder bound
                // (which only falls) gets no entry: the scatter would drop it.
                // Checked when big triangles outnumber tiles (deep overdraw of
                // large triangles); with few, the check's load costs more.
                const uint32_t zlo = early_cull ? zmin_key(t, wrap_free(t)) : 0u;
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (early_cull && ((dq >> (2 * q)) & 3u))
                    {
                        const uint32_t tq = tile00 + (uint32_t)((q >> 1) * tdx + (q & 1));
                        const uint32_t zocc_now = *(volatile uint32_t*)&a.tile_zocc[tq];
                        if (zocc_now != 0xFFFFFFFFu && zlo > min(zocc_now, 0xBF800000u))
                            dq &= ~(3u << (2 * q));
                    }
            }
            const uint32_t nz = (dq | (dq >> 1)) & 0x55u;
            const int cnt = __popc(nz);
            int cincl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const int v = __shfl_up_sync(0xffffffffu, cincl, o);
                if (lane >= (uint32_t)o) cincl += v;
            }
            const uint32_t h = (uint32_t)__shfl_sync(0xffffffffu, cincl, 31);
            if (h == 0)
                continue;
            if (h > cleft)
            {
                mark_empty();
                uint32_t nbase = 0;
                if (lane == 0)
                    nbase = atomicAdd(stripe_counter(a, stripe), kBigChunk);
                cbase = stripe_begin(a, stripe) + __shfl_sync(0xffffffffu, nbase, 0);
                cleft = kBigChunk;
            }
            uint64_t pos = cbase + (uint32_t)(cincl - cnt);
#pragma unroll
            for (int q = 0; q < 4; q++)
            {
                const uint32_t d = (dq >> (2 * q)) & 3u;
                if (!d)
                    continue;
                const uint32_t tile = tile00 + (uint32_t)((q >> 1) * tdx + (q & 1));
                atomicAdd(&a.tile_count[tile], 1u);
                if (d == kDecisionAccept && zocc != 0xFFFFFFFFu)
                    atomicMin(&a.tile_zocc[tile], zocc);
                if (pos < send)
                    a.bin_tmp[pos] = make_uint2(tile, (ri << 2) | d);
                pos++;
            }
            cbase += h;
            cleft -= h;
        }
    }
    mark_empty();
}

// -------------------------------------------------------------------------
// Exclusive scan of the per-tile counts, each rounded up to a multiple of 4
// entries so every bin starts on a 16-byte boundary, in one pass: blocks
// take consecutive ranges of kScanBlock tiles in the order they start (a
// ticket, so every range a block waits for belongs to a block already
// running) and find their offset by looking back over the published sums of
// the ranges before them (scan_status: 0 not yet, kScanAggregate | sum of
// the range, kScanPrefix | sum of everything up to the range's end).
//
// The same pass lists the raster work items: one per tile (an empty tile's
// item writes its background) plus one per further tune.item_entries entries.
// Items of at least 3/4 of that are listed from the front of the
// item array, the lighter ones from its back, and the queue hands out the
// front list first: the heavy work starts early instead of forming the tail.
__device__ __forceinline__ uint32_t padded(uint32_t c) { return (c + 3u) & ~3u; }

constexpr unsigned long long kScanAggregate = 1ull << 32;
constexpr unsigned long long kScanPrefix = 2ull << 32;
constexpr int kScanSpinLimit = 1 << 22;

// Block-wide inclusive scan of one value per thread; returns the inclusive
// value and sets `total` (all threads).
__device__ __forceinline__ uint32_t block_scan(uint32_t v, uint32_t* warp_sums, uint32_t& total)
{
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += t;
    }
    if (lane == 31)
        warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        const uint32_t w = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= (uint32_t)o) wi += t;
        }
        warp_sums[lane] = wi - w;
        if (lane == 31)
            warp_sums[32] = wi;
    }
    __syncthreads();
    total = warp_sums[32];
    return warp_sums[warp] + incl;
}

__global__ void __launch_bounds__(kScanThreads) k_scan(PassArgs a)
{
    __shared__ uint32_t warp_sums[33];
    __shared__ uint32_t s_block, s_prefix;
    if (threadIdx.x == 0)
        s_block = atomicAdd(&a.counters[8], 1u);
    __syncthreads();
    const uint32_t b = s_block;
    const uint32_t base = b * kScanBlock + threadIdx.x * kScanItems;
    uint32_t cnt[kScanItems], sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
    {
        const uint32_t i = base + k;
        cnt[k] = (i < a.total_tiles) ? a.tile_count[i] : 0u;
        sum += padded(cnt[k]);
    }
    uint32_t total;
    const uint32_t incl = block_scan(sum, warp_sums, total);
    if (threadIdx.x == 0)
    {
        uint32_t prefix = 0;
        // (a failure test makes one block keep its sums to itself)
        const bool publish = (int)b != a.tune.scan_stall_block;
        const int spin_limit = a.tune.scan_spin_limit > 0 ? a.tune.scan_spin_limit : kScanSpinLimit;
        if (b == 0)
        {
            if (publish)
                atomicExch(&a.scan_status[0], kScanPrefix | total);
        }
        else
        {
            if (publish)
                atomicExch(&a.scan_status[b], kScanAggregate | total);
            for (int j = (int)b - 1; j >= 0;)
            {
                unsigned long long st = 0;
                int spins = 0;
                do
                    st = *(volatile unsigned long long*)&a.scan_status[j];
                while (st == 0 && ++spins < spin_limit);
                if (st == 0)
                {
                    // a range never published: report it, never hang
                    atomicOr(&a.status->error, 3u);  // EDXR_ERR_TIMEOUT
                    break;
                }
                prefix += (uint32_t)st;
                if (st & kScanPrefix)
                    break;
                j--;
            }
            if (publish)
                atomicExch(&a.scan_status[b], kScanPrefix | (prefix + total));
        }
        s_prefix = prefix;
    }
    __syncthreads();
    const uint32_t prefix = s_prefix;

    // offsets, and the items of this thread's tiles.  A frame whose entries
    // did not all fit (the unsorted list or the bins overflowed) is rendered
    // again by the host; its tiles are made empty here, so no raster item
    // reads a bin with missing entries or leaves a split tile's keys behind.
    const bool dropped =
        __syncthreads_or(threadIdx.x < (uint32_t)kBinStripes &&
                         *(volatile uint32_t*)stripe_counter(a, threadIdx.x) > stripe_slots(a.bin_capacity)) != 0;
    // entries per work item; items of at least 3/4 of that are heavy
    const uint32_t E = (uint32_t)a.tune.item_entries, heavy_min = E - E / 4;
    uint32_t run = prefix + incl - sum;
    uint32_t nheavy = 0, nlight = 0;
    uint32_t start[kScanItems], n[kScanItems];
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
    {
        const uint32_t i = base + k;
        start[k] = run;
        n[k] = 0;
        if (i < a.total_tiles)
        {
            a.tile_offset[i] = run;
            uint32_t c = cnt[k];
            a.tile_count[i] = 0;  // from here on: the split tile's rastered entries
            if (dropped || (uint64_t)run + c > a.bin_capacity)
                c = 0;
            n[k] = max(1u, (c + E - 1) / E);
            // only the last item of a tile can be light
            const uint32_t light = (c - (n[k] - 1) * E) < heavy_min ? 1u : 0u;
            nlight += light;
            nheavy += n[k] - light;
            cnt[k] = c;
        }
        run += padded(cnt[k]);
    }
    // one atomic per warp and list (heavy count in the low half, light
    // count in the high half of one word: at most 32 * 4 * 2^8 and 128)
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t packed = nheavy | (nlight << 24);
    uint32_t pincl = packed;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t t = __shfl_up_sync(0xffffffffu, pincl, o);
        if (lane >= (uint32_t)o) pincl += t;
    }
    uint32_t hbase = 0, lbase = 0;
    if (lane == 31)
    {
        if (pincl & 0xFFFFFFu)
            hbase = atomicAdd(&a.counters[6], pincl & 0xFFFFFFu);
        if (pincl >> 24)
            lbase = atomicAdd(&a.counters[7], pincl >> 24);
    }
    const uint32_t pexcl = pincl - packed;
    hbase = __shfl_sync(0xffffffffu, hbase, 31) + (pexcl & 0xFFFFFFu);
    lbase = __shfl_sync(0xffffffffu, lbase, 31) + (pexcl >> 24);
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
    {
        const uint32_t i = base + k;
        if (i >= a.total_tiles)
            continue;
        const bool light = (cnt[k] - (n[k] - 1) * E) < heavy_min;
        const uint32_t heavy = n[k] - (light ? 1u : 0u);
        const uint32_t end = start[k] + cnt[k];
        const uint32_t tag = i | (n[k] > 1 ? kSplitTile : 0u);
        for (uint32_t j = 0; j < heavy; j++, hbase++)
            if (hbase < a.item_capacity)
                a.items[hbase] = make_uint4(tag, start[k] + j * E, min(end, start[k] + (j + 1) * E), 0u);
        if (light)
        {
            if (lbase < a.item_capacity)
                a.items[a.item_capacity - 1 - lbase] = make_uint4(tag, start[k] + (n[k] - 1) * E, end, 0u);
            lbase++;
        }
    }

    // the range holding the last tile has the grand total
    if (a.total_tiles > 0 && b == (a.total_tiles - 1) / kScanBlock && threadIdx.x == kScanThreads - 1)
    {
        const uint64_t grand = prefix + total;
        a.tile_offset[a.total_tiles] = (uint32_t)grand;
        // the unsorted list's stripes share the capacity: the fullest decides
        uint64_t fullest = 0, entries = 0, survivors = 0;
        for (int r = 0; r < kBinStripes; r++)
        {
            const uint32_t* c = stripe_counter(a, (uint32_t)r);
            fullest = max(fullest, (uint64_t)c[0]);
            entries += c[0];
            survivors += c[1];
        }
        const uint64_t needed = max(grand, fullest * kBinStripes);
        a.status->bins_needed = needed;
        a.status->bin_entries = entries;
        a.status->raster_tris = (uint32_t)survivors + a.counters[11];
        a.status->rtri_slots = a.total_tris + a.counters[0];
        a.status->big_tris = a.counters[2];
        if ((uint64_t)a.total_tris + a.counters[0] > a.rtri_capacity)
            atomicOr(&a.status->overflow, 2u);
        if (a.counters[4] > a.poly_capacity)
            atomicOr(&a.status->overflow, 4u);
        a.status->clipped_polys = a.counters[4];  // one polygon record per queued triangle
        if (needed > a.bin_capacity)
            atomicOr(&a.status->overflow, 1u);
        if (a.counters[2] > a.big_capacity)
            atomicOr(&a.status->overflow, 8u);
    }
}

// -------------------------------------------------------------------------
// Raster: persistent warps take work items from a queue.  An item is one
// 16x16 tile's slice of at most tune.item_entries bin entries; the warp keeps one
// 64-bit key per pixel of the tile in shared memory.  The winner of the
// reference's sequential depth test at a pixel is the fragment with the
// smallest key (depth key << 32 | submission rank term): for LEQUAL the last
// fragment with the smallest depth wins, for LESS the first.  Keys can be
// combined in any order, so the bin needs no ordering and two paths share
// the work of each group of 32 entries (one staged per lane):
//  * small entries (region of at most tune.small_region pixels): their
//    (entry, pixel) pairs are spread over the lanes, merging into the key
//    array with a shared 64-bit atomicMin;
//  * the other entries are staged as tile-relative edge equations and
//    rasterized pixel-parallel by the whole warp over their region.
// Entries whose depth lower bound is behind every pixel of the tile so far
// (the tile's hierarchical depth bound) are skipped.  The winners are then
// shaded by the same warp: directly for a tile of one item; for a tile split
// into several items, by the item that finishes last, after all of them
// merged their keys in the per-pixel key buffer.
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

// Tile-relative edge equations, barycentric numerators and region of one
// bin entry.
// With MS (several samples per pixel) it also returns G[k] = B[k] + C[k]:
// sample s sits at (o, o) from the pixel centre (see kSampleOffsets), where
// edge k changes by o * G[k]; and it keeps the quad-aligned region.
template <bool MS = false>
__device__ __forceinline__ void stage_tri(const PassArgs& a, uint32_t entry, uint32_t nr, uint32_t rank_base,
                                          int tileX, int tileY,
                                          StagedTri& s, uint32_t& zkey, int* G = nullptr)
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
    if (MS)
    {
#pragma unroll
        for (int k = 0; k < 3; k++)
            G[k] = wadd(e.B[k], e.C[k]);
    }
    // wrap-free: covered pixel centres lie in the vertices' bounding box (the
    // tight region, single sample only: an off-centre sample can be covered
    // where the centre is not), and the depth bound below holds at every
    // covered sample
    const bool wfree = wrap_free(t);
    const bool wf = !MS && wfree;
    int lx0 = 0, lx1 = 15, ly0 = 0, ly1 = 15;
    if (!accept)
    {
        // FineRasterize's quad-aligned bounding box (Rasterizer.h:132-140),
        // or only the pixels whose centre is in the vertices' bounding box
        // when no edge function can wrap (no other centre can be covered)
        const int minx = min(t.v0x, min(t.v1x, t.v2x)), maxx = max(t.v0x, max(t.v1x, t.v2x));
        const int miny = min(t.v0y, min(t.v1y, t.v2y)), maxy = max(t.v0y, max(t.v1y, t.v2y));
        // with several samples, each inside its own pixel (offsets -8..7 in
        // 1/16 pixel): the pixels the wrap-free triangle's box overlaps
        const bool box = MS && wfree;
        const int bbx0 = wf ? centre_lo(minx) : box ? minx >> 4 : (minx >> 4) & ~1;
        const int bbx1 = wf ? centre_hi(maxx) : box ? maxx >> 4 : (maxx >> 4) | 1;
        const int bby0 = wf ? centre_lo(miny) : box ? miny >> 4 : (miny >> 4) & ~1;
        const int bby1 = wf ? centre_hi(maxy) : box ? maxy >> 4 : (maxy >> 4) | 1;
        lx0 = max(0, bbx0 - (tileX << 4));
        lx1 = min(15, bbx1 - (tileX << 4));
        ly0 = max(0, bby0 - (tileY << 4));
        ly1 = min(15, bby1 - (tileY << 4));
        if (lx1 < lx0 || ly1 < ly0) { lx0 = 16; lx1 = 0; ly0 = 16; ly1 = 0; }
    }
    s.flags = (uint32_t)lx0 | ((uint32_t)lx1 << 5) | ((uint32_t)ly0 << 10) | ((uint32_t)ly1 << 15) |
              (accept ? (1u << 20) : 0u) | (bias[1] ? (1u << 21) : 0u) | (bias[2] ? (1u << 22) : 0u);
    s.invDet = t.invDet;
    s.z0 = t.z0; s.z1 = t.z1; s.z2 = t.z2;
    // submission order within the frame, offset by the frame's first input
    // triangle, so the winner's record is found from the rank alone
    s.rank = rank_base + t.order + 1u;
    zkey = zmin_key(t, wfree);
}

// Key of the fragment of staged triangle s at tile pixel (lx, ly), or false
// when the pixel is not covered (FineRasterize's edge test; trivially
// accepted entries skip it) or the depth is NaN (never passes).
__device__ __forceinline__ bool fragment_key(const StagedTri& s, int lx, int ly, bool less, uint64_t& key)
{
    // (no early exit: the lanes of a warp test different pixels, and the
    // arithmetic of an uncovered one costs the warp nothing extra)
    const uint32_t fl = s.flags;
    const int l1 = wadd(wadd(wmul(s.A1, lx), wmul(s.D1, ly)), s.K1);
    const int l2 = wadd(wadd(wmul(s.A2, lx), wmul(s.D2, ly)), s.K2);
    const int e0 = wadd(wadd(wmul(s.A0, lx), wmul(s.D0, ly)), s.K0);
    const int e1 = wadd(l1, (fl & (1u << 21)) ? -1 : 0);
    const int e2 = wadd(l2, (fl & (1u << 22)) ? -1 : 0);
    const bool inside = (fl & (1u << 20)) || (e0 | e1 | e2) >= 0;
    // TriangleSSE::CalcBarycentricCoord / GetDepth (RasterTriangle.h:324-337)
    const float L0 = fmul(__int2float_rn(l1), s.invDet);
    const float L1 = fmul(__int2float_rn(l2), s.invDet);
    const float L2 = fsub(fsub(1.0f, L0), L1);
    const float d = fadd(fadd(fmul(L0, s.z0), fmul(L1, s.z1)), fmul(L2, s.z2));
    key = ((uint64_t)depth_key(d) << 32) | (less ? s.rank : ~s.rank);
    return inside && d == d;
}

constexpr int kRasterWarps = kRasterThreads / 32;

// A staged entry padded to 80 bytes: lanes reading different entries hit
// different shared-memory banks.
struct __align__(16) StagedSlot
{
    StagedTri s;
    uint4 pad;
};

// The next work item of a persistent raster warp: after the first (item
// number = the warp's index in the grid, no claim), items first_items,
// first_items + 1, ... are claimed one at a time.
__device__ __forceinline__ uint32_t claim_item(const PassArgs& a, uint32_t first_items)
{
    uint32_t q = 0;
    if ((threadIdx.x & 31) == 0)
        q = first_items + atomicAdd(&a.counters[3], 1u);
    return __shfl_sync(0xffffffffu, q, 0);
}

// Raster triangle of the fragment with submission rank `rank` (0: none), or
// kNoTriangle.  rank - 1 = flattened input triangle * 16 + fan field: 0 for a
// triangle that was not clipped, whose record sits at its flattened index;
// piece `fan` of a clipped triangle otherwise, in slot tri_first + fan - 1
// (each clipped triangle reserves a slot per fan piece, in fan order).
__device__ __forceinline__ uint32_t raster_triangle_of(const PassArgs& a, uint32_t rank, uint32_t nr)
{
    if (rank == 0)
        return kNoTriangle;
    const uint32_t gi = (rank - 1u) >> 4, fan = (rank - 1u) & 15u;
    if (fan == 0)
        return gi < a.total_tris ? gi : kNoTriangle;
    const uint32_t ri = gi < a.total_tris ? a.tri_first[gi] + fan - 1u : kNoTriangle;
    return ri < nr ? ri : kNoTriangle;
}

// *p += v at device scope with acquire-release semantics; returns the old
// value.  A split tile's items count its rastered entries with it (see k_raster).
__device__ __forceinline__ uint32_t atomic_add_acq_rel(uint32_t* p, uint32_t v)
{
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;\n" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// Depth of raster triangle t at 1/16-pixel position (x, y)
// (RasterTriangle.h:324-337).
__device__ __forceinline__ float depth_at(const RTri& t, int x, int y, float& L0, float& L1)
{
    const Edges e = tri_edges(t);
    const int n1 = wadd(wmul(e.B[1], wsub(x, t.v2x)), wmul(e.C[1], wsub(y, t.v2y)));
    const int n2 = wadd(wmul(e.B[2], wsub(x, t.v2x)), wmul(e.C[2], wsub(y, t.v2y)));
    L0 = fmul(__int2float_rn(n1), t.invDet);
    L1 = fmul(__int2float_rn(n2), t.invDet);
    const float L2 = fsub(fsub(1.0f, L0), L1);
    return fadd(fadd(fmul(L0, t.z0), fmul(L1, t.z1)), fmul(L2, t.z2));
}

// The one write of a pixel (Renderer::FragmentProcessing / UpdateFrameBuffer,
// Renderer.cpp:272-350, shade every fragment and keep the last; only the
// winner is shaded here): its barycentrics and depth are recomputed exactly
// (RasterTriangle.h:324-337), then interpolated and shaded.  Inlined: a
// call per pixel cost more than the registers it spills in the raster loop.
struct PixelOut
{
    const RTri* rtris;
    const ClipPoly* polys;
    float4* color;
    float* depth;
    uint32_t* tri_id;
};

static __device__ __forceinline__ void write_pixel(const PixelOut a, const FrameDesc& f, uint32_t ri, uint64_t pix, int px,
                                                int py)
{
    if (ri == kNoTriangle)
    {
        a.color[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
        a.depth[pix] = 1.0f;
        a.tri_id[pix] = kNoTriangle;
        return;
    }
    const RTri t = a.rtris[ri];
    const Edges e = tri_edges(t);
    const int cx = (px << 4) + 8, cy = (py << 4) + 8;
    const int n1 = wadd(wmul(e.B[1], wsub(cx, t.v2x)), wmul(e.C[1], wsub(cy, t.v2y)));
    const int n2 = wadd(wmul(e.B[2], wsub(cx, t.v2x)), wmul(e.C[2], wsub(cy, t.v2y)));
    const float L0 = fmul(__int2float_rn(n1), t.invDet);
    const float L1 = fmul(__int2float_rn(n2), t.invDet);
    const float L2 = fsub(fsub(1.0f, L0), L1);
    const float d = fadd(fadd(fmul(L0, t.z0), fmul(L1, t.z1)), fmul(L2, t.z2));
    const float3 c = shade_fragment(f, t, a.rtris + ri, a.polys, L0, L1, px, py);
    a.color[pix] = make_float4(c.x, c.y, c.z, 1.0f);
    a.depth[pix] = d;
    a.tri_id[pix] = t.order >> 4;
}

// The per-vertex-attribute shaders (Blinn-Phong, Lambertian with or without
// albedo) at barycentrics (L0, L1) of raster triangle t: perspective-correct
// weights, the vertices' attributes, the shading model.  No call inside.
static __device__ __forceinline__ float3 shade_common(const FrameDesc& f, const RTri& t, const ClipPoly* polys,
                                                      float L0, float L1)
{
    float b0 = L0, b1 = L1;
    float b2 = fsub(fsub(1.0f, b0), b1);
    b0 = fmul(b0, t.invW0);
    b1 = fmul(b1, t.invW1);
    b2 = fmul(b2, t.invW2);
    const float invB = __frcp_rn(fadd(fadd(b0, b1), b2));
    b0 = fmul(b0, invB);
    b1 = fmul(b1, invB);
    b2 = fsub(fsub(1.0f, b0), b1);
    const ShadeVerts v = shade_verts(f, t, polys);
    return shade_model(f, lerp3(b0, v.p[0], b1, v.p[1], b2, v.p[2]), lerp3(b0, v.n[0], b1, v.n[1], b2, v.n[2]),
                       lerp3(b0, v.a[0], b1, v.a[1], b2, v.a[2]));
}

// The one write of a pixel for the per-vertex-attribute shaders: no call
// inside.
static __device__ __forceinline__ void write_pixel_fast(const PixelOut a, const FrameDesc& f, uint32_t ri,
                                                        uint64_t pix, int px, int py)
{
    if (ri == kNoTriangle)
    {
        a.color[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
        a.depth[pix] = 1.0f;
        a.tri_id[pix] = kNoTriangle;
        return;
    }
    const RTri t = a.rtris[ri];
    float L0, L1;
    const float d = depth_at(t, (px << 4) + 8, (py << 4) + 8, L0, L1);
    const float3 c = shade_common(f, t, a.polys, L0, L1);
    a.color[pix] = make_float4(c.x, c.y, c.z, 1.0f);
    a.depth[pix] = d;
    a.tri_id[pix] = t.order >> 4;
}

// A tile shaded by the FP64 or the textured shader: out of line, pixel by
// pixel, so that the common shaders' loop keeps its registers.
static __device__ __noinline__ void shade_tile_slow(const PixelOut out, const FrameDesc& f,
                                                    const unsigned long long* key, int tileX, int tileY, bool less,
                                                    uint32_t nr, const uint32_t* tri_first, uint32_t total_tris)
{
    const uint32_t lane = threadIdx.x & 31;
#pragma unroll 1
    for (int k = 0; k < 8; k++)
    {
        const int p = (int)lane + 32 * k;
        const int px = (tileX << 4) + (p & 15), py = (tileY << 4) + (p >> 4);
        if (px >= f.width || py >= f.height)
            continue;
        const uint32_t low = (uint32_t)key[p];
        const uint32_t rank = less ? low : ~low;
        uint32_t ri = kNoTriangle;
        if (rank)
        {
            // raster_triangle_of on the pass's tables
            const uint32_t gi = (rank - 1u) >> 4, fan = (rank - 1u) & 15u;
            if (gi < total_tris)
                ri = fan == 0 ? gi : tri_first[gi] + fan - 1u;
            if (ri >= nr)
                ri = kNoTriangle;
        }
        write_pixel(out, f, ri, f.pix_base + (uint64_t)py * (uint32_t)f.width + (uint32_t)px, px, py);
    }
}

template <int MinBlocks, bool SmallPath>
__global__ void __launch_bounds__(kRasterThreads, MinBlocks) k_raster(PassArgs a)
{
    __shared__ unsigned long long s_key[kRasterWarps][256];
    __shared__ StagedSlot s_tri[kRasterWarps][32];
    if (*(volatile uint32_t*)&a.status->error)
        return;  // the pass failed (see k_bin_move); every thread of the block leaves
    // ceil(65536 / w): ((p * s_recip[w]) >> 16) == p / w for 0 <= p < 256 and
    // 1 <= w <= 16, the row of pixel p of a region w pixels wide
    __shared__ uint32_t s_recip[17];
    if (threadIdx.x >= 1 && threadIdx.x <= 16)
        s_recip[threadIdx.x] = (65536u + threadIdx.x - 1u) / threadIdx.x;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long* key = s_key[warp];
    StagedSlot* staged = s_tri[warp];
    // raster-triangle slots in use: one per input triangle, then the fan pieces
    const uint32_t nr = (uint32_t)min((uint64_t)a.total_tris + *(volatile uint32_t*)&a.counters[0],
                                      (uint64_t)a.rtri_capacity);
    const uint32_t nheavy = *(volatile uint32_t*)&a.counters[6];
    const uint32_t nitems = (uint32_t)min((uint64_t)nheavy + *(volatile uint32_t*)&a.counters[7], a.item_capacity);
    const int small_region = min(a.tune.small_region, 64);
    const PixelOut out = { a.rtris, a.polys, a.color, a.depth, a.tri_id };
    // each warp's first item is its own (the heaviest ones, no claim), the
    // rest are claimed one at a time
    for (uint32_t q = blockIdx.x * kRasterWarps + warp; q < nitems; q = claim_item(a, gridDim.x * kRasterWarps))
    {
        const uint4 item = a.items[q < nheavy ? q : (uint32_t)(a.item_capacity - 1 - (q - nheavy))];
        const uint32_t tile = item.x & ~kSplitTile;
        const uint32_t fi = a.tiles_per_frame ? tile / a.tiles_per_frame
                                              : find_frame(a.frames, a.num_frames, tile,
                                                           [](const FrameDesc& f) { return f.tile_base; });
        const FrameDesc& f = a.frames[fi];
        const uint32_t lt = tile - f.tile_base;
        const int tileX = (int)(lt % (uint32_t)f.tdx), tileY = (int)(lt / (uint32_t)f.tdx);
        const bool less = f.depth_func == 1;
        // (a frame whose entries overflowed has empty items: rendered again by the host)
        bool split = (item.x & kSplitTile) != 0;
        // the item's range within the entries its bin kept (the scatter drops
        // entries hidden behind the tile's occluder)
        uint32_t e0 = item.y, e1 = item.z, kept = 0;
        if (e0 != e1)
        {
            const uint32_t bin0 = a.tile_offset[tile];
            kept = a.tile_cursor[tile];
            e1 = min(e1, bin0 + kept);
            e0 = min(e0, e1);
            if (split && e0 == e1)
            {
                if (item.y != bin0 || kept != 0)
                    continue;  // the tile's kept entries are in its other items
                split = false;  // it kept none: its first item writes the background
            }
        }
        if (e0 == e1 && !split)
        {
            // a tile with no bin entry: its background, with no key
            for (int k = 0; k < 8; k++)
            {
                const int p = (int)lane + 32 * k;
                const int px = (tileX << 4) + (p & 15), py = (tileY << 4) + (p >> 4);
                if (px < f.width && py < f.height)
                {
                    const uint64_t pix = f.pix_base + (uint64_t)py * (uint32_t)f.width + (uint32_t)px;
                    a.color[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
                    a.depth[pix] = 1.0f;
                    a.tri_id[pix] = kNoTriangle;
                }
            }
            continue;
        }

        // clear depth 1.0 with no triangle: rank term ~0 (LEQUAL) or 0 (LESS)
        const unsigned long long clear = ((unsigned long long)0xBF800000u << 32) | (less ? 0u : 0xFFFFFFFFu);
#pragma unroll
        for (int k = 0; k < 8; k++)
            key[lane + 32 * k] = clear;
        __syncwarp();
        // depth bound of the tile: the nearest triangle that covers it whole,
        // then the largest depth key of its pixels so far
        const uint32_t tzocc = min(0xBF800000u, a.tile_zocc[tile]);
        uint32_t tzmax = tzocc;

        // each chunk's bin entries load while the previous chunk is rasterized
        uint32_t next = e0 + lane < e1 ? a.bins[e0 + lane] : 0u;
        for (uint32_t c = e0; c < e1; c += 32)
        {
            const uint32_t m = min(32u, e1 - c);
            const uint32_t entry = next;
            if (c + 32 + lane < e1)
                next = a.bins[c + 32 + lane];
            int nsmall = 0;
            bool big = false;
            if (lane < m)
            {
                StagedTri s;
                uint32_t zk;
                stage_tri(a, entry, nr, f.tri_base << 4, tileX, tileY, s, zk);
                const uint32_t fl = s.flags;
                const int rx0 = fl & 31, rx1 = (fl >> 5) & 31, ry0 = (fl >> 10) & 31, ry1 = (fl >> 15) & 31;
                if (zk <= tzmax && rx0 <= rx1 && ry0 <= ry1)
                {
                    staged[lane].s = s;
                    const int area = (rx1 - rx0 + 1) * (ry1 - ry0 + 1);
                    if (SmallPath && !(fl & (1u << 20)) && area <= small_region)
                        nsmall = area;
                    else
                        big = true;
                }
            }
            // Small entries: their (entry, pixel) pairs are numbered across
            // the warp and taken 32 at a time, so lanes do not idle while
            // one lane walks a larger region.
            int incl = nsmall;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (uint32_t)o) incl += v;
            }
            const int pairs = __shfl_sync(0xffffffffu, incl, 31);
            __syncwarp();
            for (int base = 0; base < pairs; base += 32)
            {
                const int p = base + (int)lane;
                // owner: the first lane whose inclusive count exceeds p
                int j = 0;
#pragma unroll
                for (int st = 16; st >= 1; st >>= 1)
                {
                    const int v = __shfl_sync(0xffffffffu, incl, j + st - 1);
                    if (v <= p) j += st;
                }
                const int first = __shfl_sync(0xffffffffu, incl - nsmall, j);
                if (p < pairs)
                {
                    const StagedTri s = staged[j].s;
                    const uint32_t fl = s.flags;
                    const int rx0 = fl & 31, rx1 = (fl >> 5) & 31, ry0 = (fl >> 10) & 31;
                    const int rw = rx1 - rx0 + 1, local = p - first;
                    const int dy = (int)(((uint32_t)local * s_recip[rw]) >> 16);
                    const int x = rx0 + local - dy * rw, y = ry0 + dy;
                    uint64_t k;
                    // a plain read first: most fragments of deep overdraw lose
                    const bool hit = fragment_key(s, x, y, less, k);
                    const unsigned long long cur = key[y * 16 + x];
                    if (hit && k < cur)
                        atomicMin(&key[y * 16 + x], (unsigned long long)k);
                }
            }
            // Other entries: the whole warp over each region in turn.
            uint32_t todo = __ballot_sync(0xffffffffu, big);
            __syncwarp();
            while (todo)
            {
                const int j = __ffs(todo) - 1;
                todo &= todo - 1u;
                const StagedTri s = staged[j].s;
                const uint32_t fl = s.flags;
                const int rx0 = fl & 31, rx1 = (fl >> 5) & 31, ry0 = (fl >> 10) & 31, ry1 = (fl >> 15) & 31;
                const int rw = rx1 - rx0 + 1, area = rw * (ry1 - ry0 + 1);
                const uint32_t inv = s_recip[rw];
                // each pixel of the region belongs to one lane for this entry
                for (int p = (int)lane; p < area; p += 32)
                {
                    const int dy = (int)(((uint32_t)p * inv) >> 16);
                    const int x = rx0 + p - dy * rw, y = ry0 + dy;
                    uint64_t k;
                    const bool hit = fragment_key(s, x, y, less, k);
                    const unsigned long long cur = key[y * 16 + x];
                    if (hit && k < cur)
                        key[y * 16 + x] = k;
                }
                __syncwarp();
            }
            if (c + 32 < e1)
            {
                uint32_t mz = 0;
#pragma unroll
                for (int k = 0; k < 8; k++)
                    mz = max(mz, (uint32_t)(key[lane + 32 * k] >> 32));
                tzmax = min(tzocc, __reduce_max_sync(0xffffffffu, mz));
            }
        }

        // A tile split into several items merges its keys in the key buffer;
        // the item that finishes last (the one whose entries bring the tile's
        // rastered count, zeroed by the scan, to the entries its bin kept)
        // shades the tile.
        bool shade = true;
        if (split)
        {
#pragma unroll
            for (int k = 0; k < 8; k++)
            {
                const int p = (int)lane + 32 * k;
                const int px = (tileX << 4) + (p & 15), py = (tileY << 4) + (p >> 4);
                const unsigned long long kk = key[p];
                if (px < f.width && py < f.height && kk < clear)
                    atomicMax(&a.keybuf[f.pix_base + (uint64_t)py * (uint32_t)f.width + (uint32_t)px], ~kk);
            }
            // The count is one acquire-release atomic: the lanes' merges
            // happen before it (warp barrier, then lane 0's release), and
            // the item that completes the tile acquires every other item's
            // merges before it reads them back.
            __syncwarp();
            uint32_t done = 0;
            if (lane == 0)
                done = atomic_add_acq_rel(&a.tile_count[tile], e1 - e0) + (e1 - e0);
            shade = __shfl_sync(0xffffffffu, done, 0) == kept;
            __syncwarp();  // lane 0's acquire, then every lane's reads
            if (shade)
            {
#pragma unroll
                for (int k = 0; k < 8; k++)
                {
                    const int p = (int)lane + 32 * k;
                    const int px = (tileX << 4) + (p & 15), py = (tileY << 4) + (p >> 4);
                    if (px < f.width && py < f.height)
                    {
                        // read and leave zero for the next pass
                        const unsigned long long m = atomicExch(
                            &a.keybuf[f.pix_base + (uint64_t)py * (uint32_t)f.width + (uint32_t)px], 0ull);
                        key[p] = m ? ~m : clear;
                    }
                }
            }
        }
        if (shade && (f.ps_kind == 1 || f.ps_kind == 4))
            shade_tile_slow(out, f, key, tileX, tileY, less, nr, a.tri_first, a.total_tris);
        else if (shade)
        {
#pragma unroll 1
            for (int k = 0; k < 8; k++)
            {
                const int p = (int)lane + 32 * k;
                const int px = (tileX << 4) + (p & 15), py = (tileY << 4) + (p >> 4);
                const uint32_t low = (uint32_t)key[p];
                const uint32_t ri = raster_triangle_of(a, less ? low : ~low, nr);
                if (px < f.width && py < f.height)
                    write_pixel_fast(out, f, ri, f.pix_base + (uint64_t)py * (uint32_t)f.width + (uint32_t)px, px, py);
            }
        }
        __syncwarp();
    }
}

// -------------------------------------------------------------------------
// Multisampling (Renderer::SetMSAAMode, Renderer.cpp:94-98).
//
// FrameBuffer::MultiSampleOffsets (FrameBuffer.cpp:107-191): the reference's
// table of 1/16-pixel sample offsets per sample-count log2.  Its rasterizer
// reads sample s as `const Vector2i& sampleOffset = MultiSampleOffsets[level]
// [2 * s]` (Rasterizer.h:247, 382): the int goes through Vector2i's scalar
// constructor, so the sample sits at (o, o) with o = table[level][2 s].
__constant__ int kSampleOffsets[kMaxMsaaLog2 + 1][64] = {
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

__device__ __forceinline__ int sample_offset(int level, int s) { return kSampleOffsets[level][2 * s]; }

// Key of sample s (offset o) of staged triangle st at tile pixel (lx, ly):
// FineRasterize_MultiSample / TrivialAcceptTriangle_MultiSample
// (Rasterizer.h:202-300, 355-415): the biased pixel-centre edge values plus
// o * G decide coverage (accepted entries skip the test), the barycentrics
// and depth come from the unbiased values at the sample.
__device__ __forceinline__ bool sample_key(const StagedTri& st, const int* G, int lx, int ly, int o, bool less,
                                           uint64_t& key)
{
    // (no early exit: lanes of a warp test different samples, and the
    // arithmetic of an uncovered one costs the warp nothing extra)
    const uint32_t fl = st.flags;
    const int l1 = wadd(wadd(wadd(wmul(st.A1, lx), wmul(st.D1, ly)), st.K1), wmul(o, G[1]));
    const int l2 = wadd(wadd(wadd(wmul(st.A2, lx), wmul(st.D2, ly)), st.K2), wmul(o, G[2]));
    const int e0 = wadd(wadd(wadd(wmul(st.A0, lx), wmul(st.D0, ly)), st.K0), wmul(o, G[0]));
    const int e1 = wadd(l1, (fl & (1u << 21)) ? -1 : 0);
    const int e2 = wadd(l2, (fl & (1u << 22)) ? -1 : 0);
    const bool inside = (fl & (1u << 20)) || (e0 | e1 | e2) >= 0;
    const float L0 = fmul(__int2float_rn(l1), st.invDet);
    const float L1 = fmul(__int2float_rn(l2), st.invDet);
    const float L2 = fsub(fsub(1.0f, L0), L1);
    const float d = fadd(fadd(fmul(L0, st.z0), fmul(L1, st.z1)), fmul(L2, st.z2));
    key = ((uint64_t)depth_key(d) << 32) | (less ? st.rank : ~st.rank);
    return inside && d == d;
}

// Float -> 8 bits as Color4b::FromFloats: clamp, scale by 255, round half up.
__device__ __forceinline__ uint32_t to_byte(float v)
{
    v = fminf(fmaxf(v, 0.0f), 1.0f);
    return (uint32_t)fadd(fmul(v, 255.0f), 0.5f);
}


// The output of one pixel with S samples: per sample the winner's id and its
// depth at the sample; the colour is the reference's resolve
// (FrameBuffer::Resolve, FrameBuffer.cpp:70-87): each sample stores its
// winner's colour shaded at the pixel centre as 8 bits (Renderer.cpp:
// 295-350), the samples are averaged in float (alpha 1 per covered sample,
// 0 for the clear value).  Samples that share a winner share its shading.
// The winners come from the pixel's keys (key[s * 256], shared memory), read
// sample by sample.  Common: the per-vertex-attribute shaders, inline (no
// call); otherwise shade_fragment (the FP64 and textured shaders out of line).
template <bool Common>
static __device__ __forceinline__ void write_pixel_ms(const PassArgs& a, const FrameDesc& f,
                                                   const unsigned long long* key, bool less, uint32_t nr, int S,
                                                   uint64_t pix, int px, int py)
{
    const int level = a.msaa_log2;
    const uint64_t plane = a.total_pixels;
    float acc[4] = { 0.f, 0.f, 0.f, 0.f };
    uint32_t last = kNoTriangle;
    float cf[3] = { 0.f, 0.f, 0.f };  // the winner's 8-bit colour / 255
    RTri t;                            // the record of `last`
    for (int s = 0; s < S; s++)
    {
        const uint32_t low = (uint32_t)key[s * 256];
        const uint32_t r = raster_triangle_of(a, less ? low : ~low, nr);
        if (r == kNoTriangle)
        {
            a.depth[s * plane + pix] = 1.0f;
            a.tri_id[s * plane + pix] = kNoTriangle;
            continue;
        }
        if (r != last)
        {
            t = a.rtris[r];
            float L0, L1;
            depth_at(t, (px << 4) + 8, (py << 4) + 8, L0, L1);
            const float3 c = Common ? shade_common(f, t, a.polys, L0, L1)
                                    : shade_fragment(f, t, a.rtris + r, a.polys, L0, L1, px, py);
            cf[0] = fdiv((float)to_byte(c.x), 255.0f);
            cf[1] = fdiv((float)to_byte(c.y), 255.0f);
            cf[2] = fdiv((float)to_byte(c.z), 255.0f);
            last = r;
        }
        const int o = sample_offset(level, s);
        float L0, L1;
        a.depth[s * plane + pix] = depth_at(t, (px << 4) + 8 + o, (py << 4) + 8 + o, L0, L1);
        a.tri_id[s * plane + pix] = t.order >> 4;
#pragma unroll
        for (int q = 0; q < 3; q++)
            acc[q] = fadd(acc[q], cf[q]);
        acc[3] = fadd(acc[3], 1.0f);
    }
    const float inv = fdiv(1.0f, (float)S);
    a.color[pix] = make_float4(fmul(acc[0], inv), fmul(acc[1], inv), fmul(acc[2], inv), fmul(acc[3], inv));
}

// A multisampled tile shaded by the FP64 or the textured shader: out of line,
// so that the common shaders' loop keeps its registers.  (`a` is the
// kernel's grid-constant parameter: passed by address, it is not copied.)
static __device__ __noinline__ void shade_tile_ms_slow(const PassArgs& a, const FrameDesc& f,
                                                       const unsigned long long* key, int tileX, int tileY, bool less,
                                                       uint32_t nr, int S)
{
    const uint32_t lane = threadIdx.x & 31;
#pragma unroll 1
    for (int k = 0; k < 8; k++)
    {
        const int p = (int)lane + 32 * k;
        const int px = (tileX << 4) + (p & 15), py = (tileY << 4) + (p >> 4);
        if (px >= f.width || py >= f.height)
            continue;
        write_pixel_ms<false>(a, f, key + p, less, nr, S, f.pix_base + (uint64_t)py * (uint32_t)f.width + (uint32_t)px,
                              px, py);
    }
}

// Raster with S samples per pixel: persistent warps on the same work items
// as k_raster, keys [sample][pixel] in dynamic shared memory, every entry's
// (entry, pixel) pairs spread over the lanes with a loop over the samples,
// entries behind the tile's samples skipped.  Split tiles merge per sample
// in the key buffer (S planes).

// Blocks of 4 warps (2 with 16 samples, 1 with 32); registers capped where
// shared memory lets 5 blocks share an SM (2 and 4 samples: 96 registers a
// thread), the compiler's choice where it lets 3.
template <int S>
__global__ void __launch_bounds__(128, S <= 4 ? 5 : 3) k_raster_ms(const __grid_constant__ PassArgs a)
{
    extern __shared__ unsigned long long ms_shared[];
    if (*(volatile uint32_t*)&a.status->error)
        return;  // the pass failed (see k_bin_move); every thread of the block leaves
    // ceil(65536 / w): ((p * s_recip[w]) >> 16) == p / w for 0 <= p < 256
    // and 1 <= w <= 16, the row of pixel p of a region w pixels wide
    __shared__ uint32_t s_recip[17];
    if (threadIdx.x >= 1 && threadIdx.x <= 16)
        s_recip[threadIdx.x] = (65536u + threadIdx.x - 1u) / threadIdx.x;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long* key = ms_shared + (size_t)warp * (256 * S + 32 * 10);
    StagedTri* staged = reinterpret_cast<StagedTri*>(key + 256 * S);            // 32 x 64 bytes
    int* sg = reinterpret_cast<int*>(key + 256 * S + 32 * 8);                    // 32 x 3 ints (G)
    const int level = a.msaa_log2;
    // raster-triangle slots in use: one per input triangle, then the fan pieces
    const uint32_t nr = (uint32_t)min((uint64_t)a.total_tris + *(volatile uint32_t*)&a.counters[0],
                                      (uint64_t)a.rtri_capacity);
    const uint32_t nheavy = *(volatile uint32_t*)&a.counters[6];
    const uint32_t nitems = (uint32_t)min((uint64_t)nheavy + *(volatile uint32_t*)&a.counters[7], a.item_capacity);
    const uint64_t plane = a.total_pixels;
    // each warp's first item is its own (the heaviest ones, no claim), the
    // rest are claimed one at a time
    for (uint32_t q = blockIdx.x * (blockDim.x >> 5) + warp; q < nitems;
         q = claim_item(a, gridDim.x * (blockDim.x >> 5)))
    {
        const uint4 item = a.items[q < nheavy ? q : (uint32_t)(a.item_capacity - 1 - (q - nheavy))];
        const uint32_t tile = item.x & ~kSplitTile;
        const uint32_t fi = a.tiles_per_frame ? tile / a.tiles_per_frame
                                              : find_frame(a.frames, a.num_frames, tile,
                                                           [](const FrameDesc& f) { return f.tile_base; });
        const FrameDesc& f = a.frames[fi];
        const uint32_t lt = tile - f.tile_base;
        const int tileX = (int)(lt % (uint32_t)f.tdx), tileY = (int)(lt / (uint32_t)f.tdx);
        const bool less = f.depth_func == 1;
        // (a frame whose entries overflowed has empty items: rendered again by the host)
        bool split = (item.x & kSplitTile) != 0;
        // the item's range within the entries its bin kept (the scatter drops
        // entries hidden behind the tile's occluder)
        uint32_t e0 = item.y, e1 = item.z, kept = 0;
        if (e0 != e1)
        {
            const uint32_t bin0 = a.tile_offset[tile];
            kept = a.tile_cursor[tile];
            e1 = min(e1, bin0 + kept);
            e0 = min(e0, e1);
            if (split && e0 == e1)
            {
                if (item.y != bin0 || kept != 0)
                    continue;  // the tile's kept entries are in its other items
                split = false;  // it kept none: its first item writes the background
            }
        }
        if (e0 == e1 && !split)
        {
            // a tile with no bin entry: its background, with no key
            for (int k = 0; k < 8; k++)
            {
                const int p = (int)lane + 32 * k;
                const int px = (tileX << 4) + (p & 15), py = (tileY << 4) + (p >> 4);
                if (px < f.width && py < f.height)
                {
                    const uint64_t pix = f.pix_base + (uint64_t)py * (uint32_t)f.width + (uint32_t)px;
                    a.color[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
                    for (int s = 0; s < S; s++)
                    {
                        a.depth[s * plane + pix] = 1.0f;
                        a.tri_id[s * plane + pix] = kNoTriangle;
                    }
                }
            }
            continue;
        }
        const unsigned long long clear = ((unsigned long long)0xBF800000u << 32) | (less ? 0u : 0xFFFFFFFFu);
        for (int k = (int)lane; k < 256 * S; k += 32)
            key[k] = clear;
        __syncwarp();

        // depth bound of the tile: the nearest triangle that covers it whole
        // (every sample), then the largest depth key of its samples so far
        const uint32_t tzocc = min(0xBF800000u, a.tile_zocc[tile]);
        uint32_t tzmax = tzocc;
        for (uint32_t c = e0; c < e1; c += 32)
        {
            const uint32_t m = min(32u, e1 - c);
            int area = 0;
            if (lane < m)
            {
                StagedTri st;
                uint32_t zk;
                int G[3];
                stage_tri<true>(a, a.bins[c + lane], nr, f.tri_base << 4, tileX, tileY, st, zk, G);
                const uint32_t fl = st.flags;
                const int rx0 = fl & 31, rx1 = (fl >> 5) & 31, ry0 = (fl >> 10) & 31, ry1 = (fl >> 15) & 31;
                if (zk <= tzmax && rx0 <= rx1 && ry0 <= ry1)
                {
                    staged[lane] = st;
                    sg[3 * lane] = G[0];
                    sg[3 * lane + 1] = G[1];
                    sg[3 * lane + 2] = G[2];
                    area = (rx1 - rx0 + 1) * (ry1 - ry0 + 1);
                }
            }
            // (entry, pixel) pairs numbered across the warp and taken 32 at a
            // time, each lane testing the S samples of its pixel, so lanes do
            // not idle on entries of a few pixels
            int incl = area;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (uint32_t)o) incl += v;
            }
            const int pairs = __shfl_sync(0xffffffffu, incl, 31);
            __syncwarp();
            for (int base = 0; base < pairs; base += 32)
            {
                const int p = base + (int)lane;
                // owner: the first lane whose inclusive count exceeds p
                int j = 0;
#pragma unroll
                for (int st = 16; st >= 1; st >>= 1)
                {
                    const int v = __shfl_sync(0xffffffffu, incl, j + st - 1);
                    if (v <= p) j += st;
                }
                const int first = __shfl_sync(0xffffffffu, incl - area, j);
                if (p < pairs)
                {
                    const StagedTri st = staged[j];
                    const int G[3] = { sg[3 * j], sg[3 * j + 1], sg[3 * j + 2] };
                    const uint32_t fl = st.flags;
                    const int rx0 = fl & 31, rx1 = (fl >> 5) & 31, ry0 = (fl >> 10) & 31;
                    const int rw = rx1 - rx0 + 1, local = p - first;
                    const int dy = (int)(((uint32_t)local * s_recip[rw]) >> 16);
                    const int x = rx0 + local - dy * rw, y = ry0 + dy;
#pragma unroll 4
                    for (int s = 0; s < S; s++)
                    {
                        uint64_t k;
                        unsigned long long* slot = &key[s * 256 + y * 16 + x];
                        const bool hit = sample_key(st, G, x, y, sample_offset(level, s), less, k);
                        const unsigned long long cur = *slot;
                        if (hit && k < cur)
                            atomicMin(slot, (unsigned long long)k);
                    }
                }
            }
            __syncwarp();
            if (c + 32 < e1)
            {
                uint32_t mz = 0;
                for (int k = (int)lane; k < 256 * S; k += 32)
                    mz = max(mz, (uint32_t)(key[k] >> 32));
                tzmax = min(tzocc, __reduce_max_sync(0xffffffffu, mz));
            }
        }

        bool shade = true;
        if (split)
        {
            for (int k = (int)lane; k < 256 * S; k += 32)
            {
                const int s = k >> 8, p = k & 255;
                const int px = (tileX << 4) + (p & 15), py = (tileY << 4) + (p >> 4);
                const unsigned long long kk = key[k];
                if (px < f.width && py < f.height && kk < clear)
                    atomicMax(&a.keybuf[s * plane + f.pix_base + (uint64_t)py * (uint32_t)f.width + (uint32_t)px], ~kk);
            }
            // acquire-release count, as in k_raster
            __syncwarp();
            uint32_t done = 0;
            if (lane == 0)
                done = atomic_add_acq_rel(&a.tile_count[tile], e1 - e0) + (e1 - e0);
            shade = __shfl_sync(0xffffffffu, done, 0) == kept;
            __syncwarp();  // lane 0's acquire, then every lane's reads
            if (shade)
            {
                for (int k = (int)lane; k < 256 * S; k += 32)
                {
                    const int s = k >> 8, p = k & 255;
                    const int px = (tileX << 4) + (p & 15), py = (tileY << 4) + (p >> 4);
                    if (px < f.width && py < f.height)
                    {
                        const unsigned long long m = atomicExch(
                            &a.keybuf[s * plane + f.pix_base + (uint64_t)py * (uint32_t)f.width + (uint32_t)px], 0ull);
                        key[k] = m ? ~m : clear;
                    }
                }
                __syncwarp();
            }
        }
        if (shade && (f.ps_kind == 1 || f.ps_kind == 4))
            shade_tile_ms_slow(a, f, key, tileX, tileY, less, nr, S);
        else if (shade)
        {
#pragma unroll 1
            for (int k = 0; k < 8; k++)
            {
                const int p = (int)lane + 32 * k;
                const int px = (tileX << 4) + (p & 15), py = (tileY << 4) + (p >> 4);
                if (px >= f.width || py >= f.height)
                    continue;
                write_pixel_ms<true>(a, f, key + p, less, nr, S,
                                     f.pix_base + (uint64_t)py * (uint32_t)f.width + (uint32_t)px, px, py);
            }
        }
        __syncwarp();
    }
}

// Warps per block and dynamic shared memory of k_raster_ms with S samples.
static int ms_warps(int S) { return S <= 8 ? 4 : (S == 16 ? 2 : 1); }
static size_t ms_smem(int S) { return (size_t)ms_warps(S) * (256 * S + 32 * 10) * sizeof(unsigned long long); }

// -------------------------------------------------------------------------
// Renderer::GetBackBuffer compatibility: RGBA8, bottom-up (FrameBuffer.cpp:41).
__global__ void k_back_buffer(const float4* color, uchar4* out, int width, int height)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= width * height)
        return;
    const int x = i % width, y = i / width;
    const float4 c = color[i];
    // Color4b::FromFloats for one sample (alpha 1 or 0), Color4b(Color) of
    // the resolve with several (alpha = covered share)
    out[(size_t)(height - 1 - y) * width + x] =
        make_uchar4(to_byte(c.x), to_byte(c.y), to_byte(c.z), to_byte(c.w));
}

// -------------------------------------------------------------------------

// Raster variants: 0 and 1 carry the triangle-parallel path (3 blocks per SM,
// whose 85 registers a thread hold the shading epilogue without spills / 5
// blocks per SM); 2 is pixel-parallel only, capped for 6.
static int raster_occupancy(int variant)
{
    static int per_sm[3] = { 0, 0, 0 };
    if (!per_sm[variant])
    {
        cudaError_t e;
        if (variant == 0)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[0], k_raster<3, true>, kRasterThreads, 0);
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

// Resident blocks per SM of k_raster_ms with 2^level samples (the dynamic
// shared-memory limit raised first).
template <int S>
static int ms_occupancy_of()
{
    int n = 0;
    if (cudaFuncSetAttribute(k_raster_ms<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ms_smem(S)) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_raster_ms<S>, 32 * ms_warps(S), ms_smem(S)) !=
            cudaSuccess ||
        n < 1)
        n = 1;
    return n;
}

static int ms_occupancy(int level)
{
    static int per_sm[kMaxMsaaLog2 + 1] = {};
    if (!per_sm[level])
    {
        switch (level)
        {
        case 1: per_sm[1] = ms_occupancy_of<2>(); break;
        case 2: per_sm[2] = ms_occupancy_of<4>(); break;
        case 3: per_sm[3] = ms_occupancy_of<8>(); break;
        case 4: per_sm[4] = ms_occupancy_of<16>(); break;
        default: per_sm[5] = ms_occupancy_of<32>(); break;
        }
    }
    return per_sm[level];
}

void prepare_kernels()
{
    raster_occupancy(0);
    raster_occupancy(1);
    raster_occupancy(2);
    for (int level = 1; level <= kMaxMsaaLog2; level++)
        ms_occupancy(level);
}

Tuning default_tuning()
{
    Tuning t;
    t.small_region = 32;
    t.raster_variant = 1;
    t.bin_blocks_per_sm = 8;
    t.raster_blocks_per_sm = 0;
    t.item_entries = (int)kItemEntries;
    t.scan_stall_block = -1;
    t.scan_spin_limit = 0;
    return t;
}

cudaError_t launch_pipeline(const PassArgs& a, cudaStream_t s, cudaEvent_t* ev)
{
    const int sms = a.num_sms > 0 ? a.num_sms : 148;
    const uint32_t nscan = scan_blocks(a.total_tiles);
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(ev[i], s);
    };
    mark(0);
    const uint32_t clear_items = max(a.total_tiles + 1, a.vrecs ? a.total_vertices : 0u);
    k_clear<<<(clear_items + 255) / 256 + 1, 256, 0, s>>>(a);
    mark(1);
    if (a.total_tris)
    {
        k_setup<<<(a.total_tris + 255) / 256, 256, 0, s>>>(a);
        k_clip<<<sms * 8, kClipThreads, 0, s>>>(a);
    }
    k_bin_big<<<sms * 4, 256, 0, s>>>(a);
    mark(2);
    k_scan<<<nscan, kScanThreads, 0, s>>>(a);
    mark(3);
    k_bin_move<<<sms * (a.tune.bin_blocks_per_sm > 0 ? a.tune.bin_blocks_per_sm : 8), 256, 0, s>>>(a);
    mark(4);
    if (a.msaa_log2 > 0)
    {
        const int level = min(a.msaa_log2, kMaxMsaaLog2), S = 1 << level;
        const int blocks = sms * ms_occupancy(level), threads = 32 * ms_warps(S);
        switch (level)
        {
        case 1: k_raster_ms<2><<<blocks, threads, ms_smem(2), s>>>(a); break;
        case 2: k_raster_ms<4><<<blocks, threads, ms_smem(4), s>>>(a); break;
        case 3: k_raster_ms<8><<<blocks, threads, ms_smem(8), s>>>(a); break;
        case 4: k_raster_ms<16><<<blocks, threads, ms_smem(16), s>>>(a); break;
        default: k_raster_ms<32><<<blocks, threads, ms_smem(32), s>>>(a); break;
        }
    }
    else if (a.tune.raster_variant == 2)
        k_raster<6, false><<<raster_blocks(sms, a.tune), kRasterThreads, 0, s>>>(a);
    else if (a.tune.raster_variant == 1)
        k_raster<5, true><<<raster_blocks(sms, a.tune), kRasterThreads, 0, s>>>(a);
    else
        k_raster<3, true><<<raster_blocks(sms, a.tune), kRasterThreads, 0, s>>>(a);
    mark(5);
    return cudaGetLastError();
}

int kernels_per_pass(const PassArgs& a)
{
    return 5 + (a.total_tris ? 2 : 0);
}

__global__ void k_mip_level(const float4* src, int sw, int sh, float4* dst, int dw, int dh)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= dw * dh)
        return;
    const int x = i % dw, y = i / dw;
    const int x0 = min(2 * x, sw - 1), x1 = min(2 * x + 1, sw - 1);
    const int y0 = min(2 * y, sh - 1), y1 = min(2 * y + 1, sh - 1);
    const float4 a = src[(size_t)y0 * sw + x0], b = src[(size_t)y0 * sw + x1];
    const float4 c = src[(size_t)y1 * sw + x0], d = src[(size_t)y1 * sw + x1];
    auto avg = [](float p, float q, float r, float t) { return fmul(fadd(fadd(fadd(p, q), r), t), 0.25f); };
    dst[i] = make_float4(avg(a.x, b.x, c.x, d.x), avg(a.y, b.y, c.y, d.y), avg(a.z, b.z, c.z, d.z),
                         avg(a.w, b.w, c.w, d.w));
}

cudaError_t launch_mip_level(const float4* src, int sw, int sh, float4* dst, int dw, int dh, cudaStream_t s)
{
    const int n = dw * dh;
    k_mip_level<<<(n + 255) / 256, 256, 0, s>>>(src, sw, sh, dst, dw, dh);
    return cudaGetLastError();
}

cudaError_t launch_back_buffer(const float4* color, uint8_t* rgba8, int width, int height, cudaStream_t s)
{
    const int n = width * height;
    k_back_buffer<<<(n + 255) / 256, 256, 0, s>>>(color, reinterpret_cast<uchar4*>(rgba8), width, height);
    return cudaGetLastError();
}

}  // namespace edxr
