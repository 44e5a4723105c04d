// C ABI of the EDXRaster GB300 pipeline (include/edxr.h): renderer object,
// device buffers, per-frame descriptors, overflow recovery and CUDA-graph
// replay of the kernel sequence.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "edxr.h"
#include "edxr_internal.h"

using namespace edxr;

namespace {

thread_local std::string g_last_error;

edxr_status fail(edxr_status s, const std::string& msg)
{
    g_last_error = msg;
    return s;
}

}  // namespace

void edxr::record_error(const char* msg) { g_last_error = msg; }

void edxr::mat_mul(const float* A, const float* B, float* C)
{
    // P * MV as Renderer.cpp:90, each entry summed left to right in float
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
        {
            float s = A[i * 4] * B[j];
            s = s + A[i * 4 + 1] * B[4 + j];
            s = s + A[i * 4 + 2] * B[8 + j];
            s = s + A[i * 4 + 3] * B[12 + j];
            C[i * 4 + j] = s;
        }
}

// Eye position MV^-1 * 0 (Renderer.cpp:289) by Gauss-Jordan in double.
bool edxr::eye_from_mv(const float* mv, double eye[3])
{
    double a[4][8];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
        {
            a[i][j] = mv[i * 4 + j];
            a[i][j + 4] = i == j ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; c++)
    {
        int piv = c;
        for (int r = c + 1; r < 4; r++)
            if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (a[piv][c] == 0.0)
            return false;
        if (piv != c)
            for (int j = 0; j < 8; j++) std::swap(a[c][j], a[piv][j]);
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
    return true;
}

void edxr::frame_camera(FrameDesc& f, const float mv[16], const float proj[16], const float raster[16])
{
    mat_mul(proj, mv, f.mvp);
    std::memcpy(f.raster, raster, sizeof(f.raster));
    if (!eye_from_mv(mv, f.eye_d))
        f.eye_d[0] = f.eye_d[1] = f.eye_d[2] = 0.0;
    for (int q = 0; q < 3; q++)
        f.eye[q] = (float)f.eye_d[q];
    // 2D affine inverse of the raster matrix's x/y rows
    const double a = raster[0], b = raster[1], c = raster[3];
    const double d = raster[4], e = raster[5], g = raster[7];
    const double det = a * e - b * d;
    if (det != 0.0)
    {
        f.ndc_from_raster_d[0] = e / det;
        f.ndc_from_raster_d[1] = -b / det;
        f.ndc_from_raster_d[2] = (b * g - e * c) / det;
        f.ndc_from_raster_d[3] = -d / det;
        f.ndc_from_raster_d[4] = a / det;
        f.ndc_from_raster_d[5] = (d * c - a * g) / det;
        for (int q = 0; q < 6; q++)
        {
            f.ndc_from_raster[q] = (float)f.ndc_from_raster_d[q];
            f.ndc_from_raster_lo[q] = (float)(f.ndc_from_raster_d[q] - (double)f.ndc_from_raster[q]);
        }
    }
}

void edxr::frame_mesh(FrameDesc& f, const edxr_mesh& m, uint32_t width, uint32_t height)
{
    f.positions = static_cast<const char*>(m.positions);
    f.normals = static_cast<const char*>(m.normals);
    f.albedo = static_cast<const char*>(m.albedo);
    f.uvs = static_cast<const char*>(m.uvs);
    f.indices = m.indices;
    f.pos_stride = m.position_stride;
    f.nrm_stride = m.normal_stride;
    f.alb_stride = m.albedo_stride;
    f.uv_stride = m.uv_stride;
    f.nv = m.num_vertices;
    f.nt = m.num_triangles;
    f.width = (int)width;
    f.height = (int)height;
    f.tdx = (int)((width + kTileSize - 1) >> kTileLog2);
    f.tdy = (int)((height + kTileSize - 1) >> kTileLog2);
    f.tdx32 = (int)((width + 31) >> 5);
    f.tdy32 = (int)((height + 31) >> 5);
}

void edxr::frame_shading(FrameDesc& f, int ps_kind, const float light[3], float ks, float shininess)
{
    f.ps_kind = ps_kind;
    for (int q = 0; q < 3; q++)
        f.light_raw[q] = light[q];
    const double lx = light[0], ly = light[1], lz = light[2];
    const double ln = std::sqrt(lx * lx + ly * ly + lz * lz);
    f.light[0] = (float)(lx / ln);
    f.light[1] = (float)(ly / ln);
    f.light[2] = (float)(lz / ln);
    f.ks = ks;
    f.shininess = shininess;
}

namespace {

#define EDXR_CUDA(call)                                                                        \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(e_ == cudaErrorMemoryAllocation ? EDXR_ERR_OUT_OF_MEMORY : EDXR_ERR_CUDA, \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                   \
    } while (0)

// Grow-only device allocation.
struct DevBuf
{
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need)
    {
        if (need <= bytes)
            return cudaSuccess;
        if (ptr)
            cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&ptr, need);
        if (e == cudaSuccess)
            bytes = need;
        return e;
    }
    // as ensure, and a new allocation starts zeroed (in stream order)
    cudaError_t ensure_zeroed(size_t need, cudaStream_t s)
    {
        if (need <= bytes)
            return cudaSuccess;
        cudaError_t e = ensure(need);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(ptr, 0, need, s);
        return e;
    }
    void release()
    {
        if (ptr)
            cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <typename T> T* as() const { return static_cast<T*>(ptr); }
};

struct Camera
{
    float mv[16], proj[16], raster[16];
    bool set = false;
};

struct Shading
{
    int ps_kind = EDXR_PS_BLINN_PHONG;
    edxr_shader_params p = { { 1.0f, 1.0f, -1.0f }, 0.5f, 32.0f };
};

struct MeshStage
{
    DevBuf pos, nrm, alb, uv, tid, idx;
};

}  // namespace

struct edxr_renderer
{
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    uint32_t width = 0, height = 0;
    // RenderStates::DefaultSettings (RenderStates.h:55-61): LEQUAL, hierarchical, one sample, trilinear
    edxr_state state = { EDXR_DEPTH_LEQUAL, 1, 0, EDXR_FILTER_TRILINEAR };
    Shading shading;
    Camera cam;

    DevBuf frames, frame_of_block, rtris, polys, clip_list, tile_count, tile_offset, tile_cursor, tile_zocc, bins, bin_tmp,
        big_list, counters,
        status;
    DevBuf color, depth, tri_id, back8, diff_scratch, tri_first, items, keybuf, vrecs;
    // texture slots (edxr_set_textures): descriptors and the texel pool with mip chains
    DevBuf tex_desc, tex_texels;
    uint32_t num_textures = 0;
    uint64_t bin_capacity = 0, rtri_cap = 0, poly_cap = 0, big_cap = 0;
    uint64_t debug_cap = 0;  // EDXR_DEBUG_CAPACITY: tiny starting capacities (tests)
    std::vector<MeshStage> stage;
    FrameDesc* frames_host = nullptr;  // pinned
    size_t frames_host_cap = 0;
    DeviceStatus* status_host = nullptr;  // pinned
    cudaEvent_t done = nullptr;

    // the last pass, for synchronize / overflow recovery
    PassArgs last = {};
    bool pending = false;
    uint32_t last_frames = 0, out_width = 0, out_height = 0, last_samples = 1;
    uint32_t rerenders = 0;
    uint8_t* back_host = nullptr;  // pinned, GetBackBuffer's RGBA8 copy
    size_t back_host_cap = 0;

    // CUDA graph of the kernel sequence, replayed while the pass layout is unchanged
    bool use_graphs = true;
    cudaGraphExec_t graph = nullptr;
    PassArgs graph_args = {};
    PassArgs prev_args = {};
    bool has_prev_args = false;

    // stage timing
    bool profiling = false;
    cudaEvent_t stage_ev[kStageEvents] = {};

    Tuning tuning = default_tuning();
    uint32_t bins_per_tri = 2;
};

namespace {

bool same_args(const PassArgs& a, const PassArgs& b) { return std::memcmp(&a, &b, sizeof(PassArgs)) == 0; }

cudaError_t run_pass(edxr_renderer* r, const PassArgs& a)
{
    if (r->profiling)
        return launch_pipeline(a, r->stream, r->stage_ev);
    if (!r->use_graphs || r->stream == nullptr)
        return launch_pipeline(a, r->stream);
    if (r->graph && same_args(a, r->graph_args))
        return cudaGraphLaunch(r->graph, r->stream);
    // Capture only once the same pass layout repeats: a caller that changes
    // meshes every frame gets direct launches instead of a capture per frame.
    const bool repeat = r->has_prev_args && same_args(a, r->prev_args);
    r->prev_args = a;
    r->has_prev_args = true;
    if (!repeat)
        return launch_pipeline(a, r->stream);
    if (r->graph)
    {
        cudaGraphExecDestroy(r->graph);
        r->graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess)
        return launch_pipeline(a, r->stream);
    cudaError_t le = launch_pipeline(a, r->stream);
    e = cudaStreamEndCapture(r->stream, &g);
    if (le != cudaSuccess || e != cudaSuccess)
    {
        if (g) cudaGraphDestroy(g);
        return le != cudaSuccess ? le : e;
    }
    e = cudaGraphInstantiate(&r->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
    {
        r->graph = nullptr;
        return launch_pipeline(a, r->stream);
    }
    r->graph_args = a;
    return cudaGraphLaunch(r->graph, r->stream);
}

edxr_status check_mesh(const edxr_mesh* m)
{
    if (!m)
        return fail(EDXR_ERR_INVALID_ARG, "mesh is NULL");
    if (m->num_triangles > 0 && (!m->positions || !m->indices))
        return fail(EDXR_ERR_INVALID_ARG, "mesh positions and indices are required");
    if (m->num_triangles >= (1u << 28))
        return fail(EDXR_ERR_INVALID_ARG, "more than 2^28 triangles in one mesh");
    if (m->memory != EDXR_MEMORY_HOST && m->memory != EDXR_MEMORY_DEVICE)
        return fail(EDXR_ERR_INVALID_ARG, "mesh memory must be EDXR_MEMORY_HOST or EDXR_MEMORY_DEVICE");
    if (m->positions && m->position_stride < 12)
        return fail(EDXR_ERR_INVALID_ARG, "position stride below 12 bytes");
    if (m->normals && m->normal_stride < 12)
        return fail(EDXR_ERR_INVALID_ARG, "normal stride below 12 bytes");
    if (m->albedo && m->albedo_stride < 12)
        return fail(EDXR_ERR_INVALID_ARG, "albedo stride below 12 bytes");
    if (m->uvs && m->uv_stride < 8)
        return fail(EDXR_ERR_INVALID_ARG, "uv stride below 8 bytes");
    // Index range (the reference asserts it, InputBuffer.h:177) is checked by
    // the setup kernel for host and device meshes alike; a bad index makes the
    // frame fail with EDXR_ERR_INVALID_ARG at synchronisation.
    return EDXR_OK;
}

// Device address of host memory the GPU reads in place (page-locked memory
// mapped into the device's address space, reached over NVLink-C2C), or NULL.
const void* device_view(const void* p)
{
    if (!p)
        return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess)
    {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// Copy a host mesh to device staging buffers; returns a device-memory mesh.
// Positions and indices, which the vertex stage, setup and clipping read
// whole, are copied.  The shading-only arrays (normals, albedo; texture
// coordinates and texture ids for the textured shader, the one that samples
// them) are read in place when they are page-locked: only the lines of the
// winning triangles' vertices then cross the host link.  Either way the
// caller keeps the arrays unchanged until the frame completes.
edxr_status stage_mesh(edxr_renderer* r, size_t slot, const edxr_mesh* in, edxr_mesh* out, bool textured = false)
{
    *out = *in;
    if (in->memory == EDXR_MEMORY_DEVICE)
        return EDXR_OK;
    if (r->stage.size() <= slot)
        r->stage.resize(slot + 1);
    MeshStage& s = r->stage[slot];
    const size_t nv = in->num_vertices;
    auto copy = [&](DevBuf& buf, const void* src, uint32_t stride, size_t elem, const void** dst, uint32_t* dst_stride) -> edxr_status {
        if (!src)
            return EDXR_OK;
        if (&buf != &s.pos)
        {
            if (const void* view = device_view(src))
            {
                *dst = view;
                *dst_stride = stride;
                return EDXR_OK;
            }
        }
        EDXR_CUDA(buf.ensure(nv * stride > 0 ? nv * stride : 16));
        if (nv)
            EDXR_CUDA(cudaMemcpyAsync(buf.ptr, src, (nv - 1) * (size_t)stride + elem, cudaMemcpyHostToDevice, r->stream));
        *dst = buf.ptr;
        *dst_stride = stride;
        return EDXR_OK;
    };
    edxr_status st;
    if ((st = copy(s.pos, in->positions, in->position_stride, 12, &out->positions, &out->position_stride))) return st;
    if ((st = copy(s.nrm, in->normals, in->normal_stride, 12, &out->normals, &out->normal_stride))) return st;
    if ((st = copy(s.alb, in->albedo, in->albedo_stride, 12, &out->albedo, &out->albedo_stride))) return st;
    if (textured)
    {
        if ((st = copy(s.uv, in->uvs, in->uv_stride, 8, &out->uvs, &out->uv_stride))) return st;
        if (const void* view = device_view(in->texture_ids))
            out->texture_ids = static_cast<const uint32_t*>(view);
        else if (in->texture_ids)
        {
            const size_t tb = 4ull * in->num_triangles;
            EDXR_CUDA(s.tid.ensure(tb > 0 ? tb : 16));
            if (tb)
                EDXR_CUDA(cudaMemcpyAsync(s.tid.ptr, in->texture_ids, tb, cudaMemcpyHostToDevice, r->stream));
            out->texture_ids = s.tid.as<uint32_t>();
        }
    }
    else
    {
        out->uvs = nullptr;
        out->uv_stride = 0;
        out->texture_ids = nullptr;
    }
    const size_t ib = 12ull * in->num_triangles;
    EDXR_CUDA(s.idx.ensure(ib > 0 ? ib : 16));
    if (ib)
        EDXR_CUDA(cudaMemcpyAsync(s.idx.ptr, in->indices, ib, cudaMemcpyHostToDevice, r->stream));
    out->indices = s.idx.as<uint32_t>();
    out->memory = EDXR_MEMORY_DEVICE;
    return EDXR_OK;
}

void fill_frame(FrameDesc& f, const edxr_mesh& m, const Camera& cam, const Shading& sh, int depth_func,
                int hierarchical, uint32_t width, uint32_t height, const edxr_renderer* r)
{
    std::memset(&f, 0, sizeof(f));
    f.tex_ids = m.texture_ids;
    f.textures = r->tex_desc.as<TexDesc>();
    f.texels = r->tex_texels.as<float4>();
    f.num_textures = r->num_textures;
    f.tex_filter = r->state.texture_filter;
    frame_mesh(f, m, width, height);
    f.depth_func = depth_func;
    f.hierarchical = hierarchical ? 1 : 0;
    frame_camera(f, cam.mv, cam.proj, cam.raster);
    frame_shading(f, sh.ps_kind, sh.p.light, sh.p.ks, sh.p.shininess);
}

// Build the pass over `n` frames (already in r->frames_host) and launch it,
// with 2^msaa_log2 samples per pixel.
edxr_status launch_frames(edxr_renderer* r, uint32_t n, uint32_t width, uint32_t height, int msaa_log2 = 0)
{
    uint64_t tv = 0, tt = 0, tiles = 0;
    bool equal_tiles = true;
    for (uint32_t i = 0; i < n; i++)
    {
        FrameDesc& f = r->frames_host[i];
        equal_tiles = equal_tiles && (uint64_t)f.tdx * f.tdy == (uint64_t)r->frames_host[0].tdx * r->frames_host[0].tdy;
        f.vtx_base = (uint32_t)tv;
        f.tri_base = (uint32_t)tt;
        f.tile_base = (uint32_t)tiles;
        f.pix_base = (uint64_t)i * width * height;
        tv += f.nv;
        tt += f.nt;
        tiles += (uint64_t)f.tdx * f.tdy;
    }
    if (tv >= (1ull << 31) || tt >= (1ull << 28) || tiles >= (1ull << 24))
        return fail(EDXR_ERR_OVERFLOW, "pass too large: reduce the number of frames per call");
    const uint64_t pixels = (uint64_t)n * width * height;
    // Intermediate capacities start from typical needs and grow when a frame
    // reports an overflow (sync_pass renders that frame again).  The test
    // knob EDXR_DEBUG_CAPACITY starts them all tiny instead, so the first
    // frame exercises that recovery.
    // Raster-triangle slots: one per input triangle (always), then room for
    // the fan pieces of clipped triangles.
    if (r->debug_cap && r->rtri_cap == 0)
    {
        r->poly_cap = r->big_cap = r->bin_capacity = r->debug_cap;
        r->rtri_cap = tt + r->debug_cap;
    }
    else
        r->rtri_cap = std::max<uint64_t>({ r->rtri_cap, tt + (r->debug_cap ? r->debug_cap
                                                                           : std::max<uint64_t>(tt / 4, 65536)) });
    if (!r->debug_cap)
    {
        r->poly_cap = std::max<uint64_t>({ r->poly_cap, std::max<uint64_t>(tt / 16, 65536) });
        r->big_cap = std::max<uint64_t>({ r->big_cap, std::max<uint64_t>(tt / 8, 65536) });
        if (r->bin_capacity < (uint64_t)r->bins_per_tri * tt + 4 * tiles)
            r->bin_capacity = std::max<uint64_t>((uint64_t)r->bins_per_tri * tt + 4 * tiles, 1u << 20);
    }
    r->rtri_cap = std::min<uint64_t>(r->rtri_cap, 0xFFFFFFF0u);
    const uint64_t rcap = r->rtri_cap, pcap = r->poly_cap;
    const uint64_t nscan = scan_blocks(tiles);
    EDXR_CUDA(r->frames.ensure(sizeof(FrameDesc) * n));
    EDXR_CUDA(r->tri_first.ensure(4 * std::max<uint64_t>(tt, 1)));
    EDXR_CUDA(r->rtris.ensure((sizeof(RTri) + 4) * rcap));  // the records, then their depth bounds
    EDXR_CUDA(r->polys.ensure(sizeof(ClipPoly) * pcap));
    EDXR_CUDA(r->clip_list.ensure(4 * pcap));
    EDXR_CUDA(r->tile_count.ensure(4 * (tiles + 1)));
    EDXR_CUDA(r->tile_offset.ensure(4 * (tiles + 1)));
    EDXR_CUDA(r->tile_cursor.ensure(4 * (tiles + 1)));
    EDXR_CUDA(r->tile_zocc.ensure(4 * (tiles + 1)));
    EDXR_CUDA(r->bins.ensure(4 * r->bin_capacity));
    EDXR_CUDA(r->bin_tmp.ensure(8 * r->bin_capacity));
    EDXR_CUDA(r->big_list.ensure(4 * r->big_cap));
    EDXR_CUDA(r->counters.ensure(4 * kCounters + 8 * std::max<uint64_t>(nscan, 1)));  // + scan status words
    EDXR_CUDA(r->status.ensure(sizeof(DeviceStatus)));
    EDXR_CUDA(r->color.ensure(16 * std::max<uint64_t>(pixels, 1)));
    // depth and triangle ids: one plane per sample
    const uint64_t samples = 1ull << msaa_log2;
    EDXR_CUDA(r->depth.ensure(4 * samples * std::max<uint64_t>(pixels, 1)));
    EDXR_CUDA(r->tri_id.ensure(4 * samples * std::max<uint64_t>(pixels, 1)));
    EDXR_CUDA(r->keybuf.ensure_zeroed(8 * samples * std::max<uint64_t>(pixels, 1), r->stream));
    const uint64_t icap = item_capacity(tiles, r->bin_capacity, (uint32_t)r->tuning.item_entries);
    EDXR_CUDA(r->items.ensure(sizeof(uint4) * icap));
    // a vertex stage when vertices are shared (on average by at least three
    // triangle corners) and their records stay in L2 for setup to gather
    // (up to 4 Mi vertices = 64 MiB of the 126 MiB): each vertex is then
    // projected once instead of per corner
    const bool vertex_stage = tv > 0 && tv <= tt && tv <= (4u << 20);
    if (vertex_stage)
        EDXR_CUDA(r->vrecs.ensure(sizeof(int4) * tv));

    EDXR_CUDA(cudaMemcpyAsync(r->frames.ptr, r->frames_host, sizeof(FrameDesc) * n, cudaMemcpyHostToDevice, r->stream));

    PassArgs a;
    std::memset(&a, 0, sizeof(a));
    a.tune = r->tuning;
    a.frames = r->frames.as<FrameDesc>();
    a.num_frames = n;
    a.tiles_per_frame = equal_tiles && n > 1 ? (uint32_t)(tiles / n) : 0u;  // (one frame: no search)
    if (n > 1)
    {
        EDXR_CUDA(r->frame_of_block.ensure(4 * (tt / 256 + 1)));
        a.frame_of_block = r->frame_of_block.as<uint32_t>();
    }
    a.total_vertices = (uint32_t)tv;
    a.vrecs = vertex_stage ? r->vrecs.as<int4>() : nullptr;
    a.total_tris = (uint32_t)tt;
    a.total_tiles = (uint32_t)tiles;
    a.rtris = r->rtris.as<RTri>();
    a.rtri_zlo = reinterpret_cast<uint32_t*>(a.rtris + rcap);
    a.rtri_capacity = (uint32_t)std::min<uint64_t>(rcap, 0xFFFFFFFFu);
    a.polys = r->polys.as<ClipPoly>();
    a.clip_list = r->clip_list.as<uint32_t>();
    a.poly_capacity = (uint32_t)pcap;
    a.tile_count = r->tile_count.as<uint32_t>();
    a.tile_offset = r->tile_offset.as<uint32_t>();
    a.tile_cursor = r->tile_cursor.as<uint32_t>();
    a.tile_zocc = r->tile_zocc.as<uint32_t>();
    a.bins = r->bins.as<uint32_t>();
    a.bin_tmp = r->bin_tmp.as<uint2>();
    a.bin_capacity = r->bin_capacity;
    a.big_list = r->big_list.as<uint32_t>();
    a.big_capacity = (uint32_t)r->big_cap;
    a.counters = r->counters.as<uint32_t>();
    a.scan_status = reinterpret_cast<unsigned long long*>(a.counters + kCounters);
    a.status = r->status.as<DeviceStatus>();
    a.color = r->color.as<float4>();
    a.depth = r->depth.as<float>();
    a.tri_id = r->tri_id.as<uint32_t>();
    a.tri_first = r->tri_first.as<uint32_t>();
    a.items = r->items.as<uint4>();
    a.item_capacity = icap;
    a.keybuf = r->keybuf.as<unsigned long long>();
    a.total_pixels = pixels;
    a.msaa_log2 = msaa_log2;
    a.num_sms = r->num_sms;

    EDXR_CUDA(run_pass(r, a));
    EDXR_CUDA(cudaMemcpyAsync(r->status_host, r->status.ptr, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, r->stream));
    EDXR_CUDA(cudaEventRecord(r->done, r->stream));
    r->last = a;
    r->pending = true;
    r->last_frames = n;
    r->last_samples = (uint32_t)samples;
    r->out_width = width;
    r->out_height = height;
    return EDXR_OK;
}

edxr_status ensure_frames_host(edxr_renderer* r, size_t n)
{
    if (n <= r->frames_host_cap)
        return EDXR_OK;
    if (r->frames_host)
    {
        cudaEventSynchronize(r->done);
        cudaFreeHost(r->frames_host);
        r->frames_host = nullptr;
        r->frames_host_cap = 0;
    }
    EDXR_CUDA(cudaMallocHost((void**)&r->frames_host, sizeof(FrameDesc) * n));
    r->frames_host_cap = n;
    return EDXR_OK;
}

edxr_status sync_pass(edxr_renderer* r)
{
    if (!r->pending)
        return EDXR_OK;
    for (int attempt = 0;; attempt++)
    {
        EDXR_CUDA(cudaEventSynchronize(r->done));
        EDXR_CUDA(cudaGetLastError());
        const DeviceStatus st = *r->status_host;
        if (st.error)
        {
            r->pending = false;
            return fail((edxr_status)st.error, st.error == EDXR_ERR_INVALID_ARG
                                                   ? "a triangle references a vertex index out of range"
                                                   : "the device reported an error");
        }
        if (!st.overflow)
            break;
        if (attempt >= 4)
        {
            r->pending = false;
            return fail(EDXR_ERR_OVERFLOW, "intermediate buffer overflow persists after growing");
        }
        // grow what overflowed to what the frame needs and render it again
        PassArgs a = r->last;
        if (st.overflow & 2u)
        {
            r->rtri_cap = std::min<uint64_t>((uint64_t)st.rtri_slots + st.rtri_slots / 4 + 1024, 0xFFFFFFF0u);
            EDXR_CUDA(r->rtris.ensure((sizeof(RTri) + 4) * r->rtri_cap));
            a.rtris = r->rtris.as<RTri>();
            a.rtri_zlo = reinterpret_cast<uint32_t*>(a.rtris + r->rtri_cap);
            a.rtri_capacity = (uint32_t)r->rtri_cap;
        }
        if (st.overflow & 4u)
        {
            r->poly_cap = (uint64_t)st.clipped_polys + st.clipped_polys / 4 + 1024;
            EDXR_CUDA(r->polys.ensure(sizeof(ClipPoly) * r->poly_cap));
            EDXR_CUDA(r->clip_list.ensure(4 * r->poly_cap));
            a.polys = r->polys.as<ClipPoly>();
            a.clip_list = r->clip_list.as<uint32_t>();
            a.poly_capacity = (uint32_t)r->poly_cap;
        }
        if (st.overflow & 8u)
        {
            r->big_cap = (uint64_t)st.big_tris + st.big_tris / 4 + 1024;
            EDXR_CUDA(r->big_list.ensure(4 * r->big_cap));
            a.big_list = r->big_list.as<uint32_t>();
            a.big_capacity = (uint32_t)r->big_cap;
        }
        if (st.overflow & 1u)
        {
            // bins are sized from the triangles that were binned; after a
            // raster-triangle overflow the count is not final, so retry as well
            r->bin_capacity = st.bins_needed + st.bins_needed / 4 + 1024;
            EDXR_CUDA(r->bins.ensure(4 * r->bin_capacity));
            EDXR_CUDA(r->bin_tmp.ensure(8 * r->bin_capacity));
            a.bins = r->bins.as<uint32_t>();
            a.bin_tmp = r->bin_tmp.as<uint2>();
            a.bin_capacity = r->bin_capacity;
            a.item_capacity = item_capacity(a.total_tiles, r->bin_capacity, (uint32_t)r->tuning.item_entries);
            EDXR_CUDA(r->items.ensure(sizeof(uint4) * a.item_capacity));
            a.items = r->items.as<uint4>();
        }
        r->rerenders++;
        EDXR_CUDA(run_pass(r, a));
        EDXR_CUDA(cudaMemcpyAsync(r->status_host, r->status.ptr, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, r->stream));
        EDXR_CUDA(cudaEventRecord(r->done, r->stream));
        r->last = a;
    }
    r->pending = false;
    return EDXR_OK;
}

struct DeviceGuard
{
    int prev = -1;
    explicit DeviceGuard(int d)
    {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != d)
            cudaSetDevice(d);
        else
            prev = -1;
    }
    ~DeviceGuard()
    {
        if (prev >= 0)
            cudaSetDevice(prev);
    }
};

}  // namespace

extern "C" {

const char* edxr_last_error_string(void) { return g_last_error.c_str(); }

edxr_status edxr_create(edxr_renderer** out, const edxr_init* init)
{
    if (!out || !init)
        return fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (init->width == 0 || init->height == 0 || init->width > 32768 || init->height > 32768)
        return fail(EDXR_ERR_INVALID_ARG, "framebuffer size must be in [1, 32768]");
    int ndev = 0;
    EDXR_CUDA(cudaGetDeviceCount(&ndev));
    if (init->device < 0 || init->device >= ndev)
        return fail(EDXR_ERR_INVALID_ARG, "no such CUDA device");
    DeviceGuard g(init->device);
    edxr_renderer* r = new edxr_renderer();
    r->device = init->device;
    r->stream = static_cast<cudaStream_t>(init->stream);
    r->width = init->width;
    r->height = init->height;
    cudaDeviceGetAttribute(&r->num_sms, cudaDevAttrMultiProcessorCount, r->device);
    prepare_kernels();  // occupancy queries happen outside any graph capture
    if (const char* e = std::getenv("EDXR_NO_GRAPHS"))
        r->use_graphs = e[0] == '0';
    if (const char* e = std::getenv("EDXR_DEBUG_CAPACITY"))
        r->debug_cap = std::max<uint64_t>(std::strtoull(e, nullptr, 10), 4);
    cudaError_t e = cudaMallocHost((void**)&r->status_host, sizeof(DeviceStatus));
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming);
    if (e != cudaSuccess)
    {
        edxr_destroy(r);
        return fail(EDXR_ERR_CUDA, std::string("renderer setup: ") + cudaGetErrorString(e));
    }
    std::memset(r->status_host, 0, sizeof(DeviceStatus));
    *out = r;
    return EDXR_OK;
}

edxr_status edxr_destroy(edxr_renderer* r)
{
    if (!r)
        return EDXR_OK;
    DeviceGuard g(r->device);
    if (r->done)
        cudaEventSynchronize(r->done);
    if (r->graph)
        cudaGraphExecDestroy(r->graph);
    DevBuf* bufs[] = { &r->frames, &r->frame_of_block, &r->rtris, &r->polys, &r->clip_list, &r->tile_count, &r->tile_offset,
                       &r->tile_cursor, &r->tile_zocc, &r->bins, &r->bin_tmp, &r->big_list, &r->counters, &r->status, &r->color,
                       &r->depth, &r->tri_id, &r->back8, &r->diff_scratch, &r->tri_first, &r->items,
                       &r->keybuf, &r->tex_desc, &r->tex_texels, &r->vrecs };
    for (DevBuf* b : bufs)
        b->release();
    for (auto& s : r->stage)
    {
        s.pos.release(); s.nrm.release(); s.alb.release(); s.uv.release(); s.tid.release(); s.idx.release();
    }
    if (r->frames_host)
        cudaFreeHost(r->frames_host);
    if (r->status_host)
        cudaFreeHost(r->status_host);
    if (r->back_host)
        cudaFreeHost(r->back_host);
    if (r->done)
        cudaEventDestroy(r->done);
    for (int i = 0; i < kStageEvents; i++)
        if (r->stage_ev[i])
            cudaEventDestroy(r->stage_ev[i]);
    delete r;
    return EDXR_OK;
}

edxr_status edxr_resize(edxr_renderer* r, uint32_t width, uint32_t height)
{
    if (!r)
        return fail(EDXR_ERR_INVALID_ARG, "NULL renderer");
    if (width == 0 || height == 0 || width > 32768 || height > 32768)
        return fail(EDXR_ERR_INVALID_ARG, "framebuffer size must be in [1, 32768]");
    DeviceGuard g(r->device);
    edxr_status s = sync_pass(r);
    if (s != EDXR_OK)
        return s;
    r->width = width;
    r->height = height;
    return EDXR_OK;
}

edxr_status edxr_set_transform(edxr_renderer* r, const float mv[16], const float proj[16], const float raster[16])
{
    if (!r || !mv || !proj || !raster)
        return fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    std::memcpy(r->cam.mv, mv, 64);
    std::memcpy(r->cam.proj, proj, 64);
    std::memcpy(r->cam.raster, raster, 64);
    r->cam.set = true;
    return EDXR_OK;
}

edxr_status edxr_set_state(edxr_renderer* r, const edxr_state* s)
{
    if (!r || !s)
        return fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    if (s->depth_func != EDXR_DEPTH_LEQUAL && s->depth_func != EDXR_DEPTH_LESS)
        return fail(EDXR_ERR_INVALID_ARG, "unknown depth function");
    if (s->msaa_log2 < 0 || s->msaa_log2 > kMaxMsaaLog2)
        return fail(EDXR_ERR_INVALID_ARG, "msaa_log2 must be in [0, 5] (1 to 32 samples)");
    if (s->texture_filter < EDXR_FILTER_NEAREST || s->texture_filter > EDXR_FILTER_ANISOTROPIC_16X)
        return fail(EDXR_ERR_INVALID_ARG, "unknown texture filter");
    r->state = *s;
    return EDXR_OK;
}

edxr_status edxr_set_shader(edxr_renderer* r, int vs_kind, int ps_kind, const edxr_shader_params* p)
{
    if (!r)
        return fail(EDXR_ERR_INVALID_ARG, "NULL renderer");
    if (vs_kind != EDXR_VS_DEFAULT)
        return fail(EDXR_ERR_INVALID_ARG, "unknown vertex shader");
    if (ps_kind < EDXR_PS_BLINN_PHONG || ps_kind > EDXR_PS_LAMBERTIAN_TEXTURED)
        return fail(EDXR_ERR_INVALID_ARG, "unknown pixel shader");
    r->shading.ps_kind = ps_kind;
    if (p)
    {
        const double n = std::sqrt((double)p->light[0] * p->light[0] + (double)p->light[1] * p->light[1] +
                                   (double)p->light[2] * p->light[2]);
        if (!(n > 0.0) || !std::isfinite(n))
            return fail(EDXR_ERR_INVALID_ARG, "light direction must be a finite non-zero vector");
        r->shading.p = *p;
    }
    return EDXR_OK;
}

edxr_status edxr_render(edxr_renderer* r, const edxr_mesh* mesh)
{
    if (!r)
        return fail(EDXR_ERR_INVALID_ARG, "NULL renderer");
    if (!r->cam.set)
        return fail(EDXR_ERR_INVALID_ARG, "edxr_set_transform was not called");
    edxr_status s = check_mesh(mesh);
    if (s != EDXR_OK)
        return s;
    DeviceGuard g(r->device);
    if ((s = sync_pass(r)) != EDXR_OK)
        return s;
    edxr_mesh dm;
    if ((s = stage_mesh(r, 0, mesh, &dm, r->shading.ps_kind == EDXR_PS_LAMBERTIAN_TEXTURED)) != EDXR_OK)
        return s;
    if ((s = ensure_frames_host(r, 1)) != EDXR_OK)
        return s;
    cudaEventSynchronize(r->done);  // the pinned descriptor may still be in flight
    fill_frame(r->frames_host[0], dm, r->cam, r->shading, r->state.depth_func, r->state.hierarchical, r->width,
               r->height, r);
    return launch_frames(r, 1, r->width, r->height, r->state.msaa_log2);
}

edxr_status edxr_set_textures(edxr_renderer* r, const edxr_texture* textures, uint32_t count)
{
    if (!r || (count && !textures))
        return fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    uint64_t total = 0;
    std::vector<TexDesc> desc(count);
    for (uint32_t i = 0; i < count; i++)
    {
        const edxr_texture& t = textures[i];
        if (t.width == 0 || t.height == 0 || t.width > 16384 || t.height > 16384 || !t.texels ||
            (t.format != EDXR_TEXTURE_RGBA8 && t.format != EDXR_TEXTURE_RGBA32F))
            return fail(EDXR_ERR_INVALID_ARG, "texture: size must be in [1, 16384], texels non-NULL, format known");
        TexDesc& d = desc[i];
        d.width = t.width;
        d.height = t.height;
        d.levels = 1;
        d.pad = 0;
        d.base = total;
        uint32_t w = t.width, h = t.height;
        total += (uint64_t)w * h;
        while (w > 1 || h > 1)
        {
            w = std::max(1u, w >> 1);
            h = std::max(1u, h >> 1);
            total += (uint64_t)w * h;
            d.levels++;
        }
    }
    DeviceGuard g(r->device);
    edxr_status s = sync_pass(r);  // frames in flight may still sample the old set
    if (s != EDXR_OK)
        return s;
    EDXR_CUDA(cudaStreamSynchronize(r->stream));
    r->num_textures = 0;
    if (count == 0)
        return EDXR_OK;
    EDXR_CUDA(r->tex_desc.ensure(sizeof(TexDesc) * count));
    EDXR_CUDA(r->tex_texels.ensure(sizeof(float4) * total));
    float4* pool = r->tex_texels.as<float4>();
    std::vector<float4> level0;
    for (uint32_t i = 0; i < count; i++)
    {
        const edxr_texture& t = textures[i];
        const TexDesc& d = desc[i];
        const size_t n = (size_t)t.width * t.height;
        if (t.format == EDXR_TEXTURE_RGBA8)
        {
            // channel = byte / 255 (Color(Color4b), the texel conversion of
            // an 8-bit image texture)
            const uint8_t* b = static_cast<const uint8_t*>(t.texels);
            level0.resize(n);
            for (size_t k = 0; k < n; k++)
                level0[k] = make_float4(b[4 * k] / 255.0f, b[4 * k + 1] / 255.0f, b[4 * k + 2] / 255.0f,
                                        b[4 * k + 3] / 255.0f);
            EDXR_CUDA(cudaMemcpy(pool + d.base, level0.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
        }
        else
            EDXR_CUDA(cudaMemcpy(pool + d.base, t.texels, sizeof(float4) * n, cudaMemcpyHostToDevice));
        uint64_t off = d.base;
        uint32_t w = t.width, h = t.height;
        for (uint32_t l = 1; l < d.levels; l++)
        {
            const uint32_t nw = std::max(1u, w >> 1), nh = std::max(1u, h >> 1);
            EDXR_CUDA(launch_mip_level(pool + off, (int)w, (int)h, pool + off + (uint64_t)w * h, (int)nw, (int)nh,
                                       r->stream));
            off += (uint64_t)w * h;
            w = nw;
            h = nh;
        }
    }
    EDXR_CUDA(cudaMemcpyAsync(r->tex_desc.ptr, desc.data(), sizeof(TexDesc) * count, cudaMemcpyHostToDevice,
                              r->stream));
    EDXR_CUDA(cudaStreamSynchronize(r->stream));
    r->num_textures = count;
    return EDXR_OK;
}

edxr_status edxr_synchronize(edxr_renderer* r)
{
    if (!r)
        return fail(EDXR_ERR_INVALID_ARG, "NULL renderer");
    DeviceGuard g(r->device);
    return sync_pass(r);
}

edxr_status edxr_get_outputs(edxr_renderer* r, edxr_outputs* out)
{
    if (!r || !out)
        return fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    DeviceGuard g(r->device);
    edxr_status s = sync_pass(r);
    if (s != EDXR_OK)
        return s;
    if (!r->last_frames)
        return fail(EDXR_ERR_INVALID_ARG, "nothing rendered yet");
    out->color = r->color.as<float>();
    out->depth = r->depth.as<float>();
    out->triangle_id = r->tri_id.as<uint32_t>();
    out->width = r->out_width;
    out->height = r->out_height;
    out->samples = r->last_samples;
    return EDXR_OK;
}

edxr_status edxr_read_outputs(edxr_renderer* r, float* color, float* depth, uint32_t* id)
{
    if (!r)
        return fail(EDXR_ERR_INVALID_ARG, "NULL renderer");
    DeviceGuard g(r->device);
    edxr_status s = sync_pass(r);
    if (s != EDXR_OK)
        return s;
    if (!r->last_frames)
        return fail(EDXR_ERR_INVALID_ARG, "nothing rendered yet");
    const size_t n = (size_t)r->out_width * r->out_height;
    const size_t ns = n * r->last_samples;  // depth and ids: one plane per sample
    if (color) EDXR_CUDA(cudaMemcpyAsync(color, r->color.ptr, 16 * n, cudaMemcpyDeviceToHost, r->stream));
    if (depth) EDXR_CUDA(cudaMemcpyAsync(depth, r->depth.ptr, 4 * ns, cudaMemcpyDeviceToHost, r->stream));
    if (id) EDXR_CUDA(cudaMemcpyAsync(id, r->tri_id.ptr, 4 * ns, cudaMemcpyDeviceToHost, r->stream));
    EDXR_CUDA(cudaStreamSynchronize(r->stream));
    return EDXR_OK;
}

edxr_status edxr_get_back_buffer(edxr_renderer* r, const uint8_t** rgba8)
{
    if (!r || !rgba8)
        return fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    DeviceGuard g(r->device);
    edxr_status s = sync_pass(r);
    if (s != EDXR_OK)
        return s;
    if (!r->last_frames)
        return fail(EDXR_ERR_INVALID_ARG, "nothing rendered yet");
    const size_t n = (size_t)r->out_width * r->out_height;
    EDXR_CUDA(r->back8.ensure(4 * n));
    EDXR_CUDA(launch_back_buffer(r->color.as<float4>(), r->back8.as<uint8_t>(), (int)r->out_width,
                                 (int)r->out_height, r->stream));
    if (r->back_host_cap < 4 * n)
    {
        if (r->back_host)
            cudaFreeHost(r->back_host);
        r->back_host = nullptr;
        r->back_host_cap = 0;
        EDXR_CUDA(cudaMallocHost((void**)&r->back_host, 4 * n));
        r->back_host_cap = 4 * n;
    }
    EDXR_CUDA(cudaMemcpyAsync(r->back_host, r->back8.ptr, 4 * n, cudaMemcpyDeviceToHost, r->stream));
    EDXR_CUDA(cudaStreamSynchronize(r->stream));
    *rgba8 = r->back_host;
    return EDXR_OK;
}

edxr_status edxr_get_stats(edxr_renderer* r, edxr_stats* st)
{
    if (!r || !st)
        return fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    DeviceGuard g(r->device);
    edxr_status s = sync_pass(r);
    if (s != EDXR_OK)
        return s;
    st->raster_triangles = r->status_host->raster_tris;
    st->bin_entries = r->status_host->bin_entries;
    st->bin_capacity = r->bin_capacity;
    st->rerenders = r->rerenders;
    st->tile_size = kTileSize;
    st->kernels_per_pass = r->last_frames ? (uint32_t)kernels_per_pass(r->last) : 0u;
    st->clipped_polygons = r->status_host->clipped_polys;
    return EDXR_OK;
}

edxr_status edxr_set_tuning(edxr_renderer* r, const edxr_tuning* t)
{
    if (!r || !t)
        return fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    if (t->small_region < 0 || t->small_region > 256 || t->raster_variant < 0 || t->raster_variant > 2 ||
        t->bin_blocks_per_sm < 1 || t->bin_blocks_per_sm > 64 || t->raster_blocks_per_sm < 0 ||
        t->raster_blocks_per_sm > 32 || t->bin_entries_per_triangle < 1 || t->bin_entries_per_triangle > 1024 ||
        t->item_entries < 32 || t->item_entries > 1024)
        return fail(EDXR_ERR_INVALID_ARG, "tuning value out of range");
    DeviceGuard g(r->device);
    edxr_status s = sync_pass(r);
    if (s != EDXR_OK)
        return s;
    r->tuning.small_region = t->small_region;
    r->tuning.raster_variant = t->raster_variant;
    r->tuning.bin_blocks_per_sm = t->bin_blocks_per_sm;
    r->tuning.raster_blocks_per_sm = t->raster_blocks_per_sm;
    r->tuning.item_entries = t->item_entries;
    r->bins_per_tri = t->bin_entries_per_triangle;
    return EDXR_OK;
}

edxr_status edxr_debug_scan_stall(edxr_renderer* r, int block, int spin_limit)
{
    if (!r)
        return fail(EDXR_ERR_INVALID_ARG, "NULL renderer");
    if (block < -1 || spin_limit < 0)
        return fail(EDXR_ERR_INVALID_ARG, "scan stall block must be >= -1 and the spin limit >= 0");
    DeviceGuard g(r->device);
    edxr_status s = sync_pass(r);
    if (s != EDXR_OK)
        return s;
    r->tuning.scan_stall_block = block;
    r->tuning.scan_spin_limit = spin_limit;
    return EDXR_OK;
}

edxr_status edxr_get_tuning(edxr_renderer* r, edxr_tuning* t)
{
    if (!r || !t)
        return fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    t->small_region = r->tuning.small_region;
    t->raster_variant = r->tuning.raster_variant;
    t->bin_blocks_per_sm = r->tuning.bin_blocks_per_sm;
    t->raster_blocks_per_sm = r->tuning.raster_blocks_per_sm;
    t->bin_entries_per_triangle = r->bins_per_tri;
    t->item_entries = r->tuning.item_entries;
    return EDXR_OK;
}

edxr_status edxr_set_profiling(edxr_renderer* r, int enable)
{
    if (!r)
        return fail(EDXR_ERR_INVALID_ARG, "NULL renderer");
    DeviceGuard g(r->device);
    edxr_status s = sync_pass(r);
    if (s != EDXR_OK)
        return s;
    if (enable && !r->stage_ev[0])
        for (int i = 0; i < kStageEvents; i++)
            EDXR_CUDA(cudaEventCreate(&r->stage_ev[i]));
    r->profiling = enable != 0;
    return EDXR_OK;
}

edxr_status edxr_get_stage_times(edxr_renderer* r, float* ms, uint32_t* count)
{
    if (!r || !ms || !count)
        return fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    if (!r->profiling)
        return fail(EDXR_ERR_INVALID_ARG, "profiling is not enabled");
    DeviceGuard g(r->device);
    edxr_status s = sync_pass(r);
    if (s != EDXR_OK)
        return s;
    const uint32_t n = std::min<uint32_t>(*count, kStageEvents - 1);
    for (uint32_t i = 0; i < n; i++)
        EDXR_CUDA(cudaEventElapsedTime(&ms[i], r->stage_ev[i], r->stage_ev[i + 1]));
    *count = n;
    return EDXR_OK;
}

edxr_status edxr_render_batched(edxr_renderer* r, const edxr_mesh* meshes, uint32_t num_meshes,
                                const edxr_view* views, uint32_t num_views, uint32_t width, uint32_t height)
{
    if (!r || !meshes || !views || num_meshes == 0 || num_views == 0)
        return fail(EDXR_ERR_INVALID_ARG, "NULL or empty argument");
    if (width == 0 || height == 0 || width > 32768 || height > 32768)
        return fail(EDXR_ERR_INVALID_ARG, "framebuffer size must be in [1, 32768]");
    edxr_status s;
    for (uint32_t m = 0; m < num_meshes; m++)
        if ((s = check_mesh(&meshes[m])) != EDXR_OK)
            return s;
    for (uint32_t v = 0; v < num_views; v++)
    {
        if (views[v].mesh >= num_meshes)
            return fail(EDXR_ERR_INVALID_ARG, "view references a mesh out of range");
        if (views[v].ps_kind < EDXR_PS_BLINN_PHONG || views[v].ps_kind > EDXR_PS_LAMBERTIAN_TEXTURED)
            return fail(EDXR_ERR_INVALID_ARG, "unknown pixel shader in view");
        if (views[v].depth_func != EDXR_DEPTH_LEQUAL && views[v].depth_func != EDXR_DEPTH_LESS)
            return fail(EDXR_ERR_INVALID_ARG, "unknown depth function in view");
    }
    if (r->state.msaa_log2 != 0)
        return fail(EDXR_ERR_UNSUPPORTED, "the batched form renders one sample per pixel (set msaa_log2 to 0)");
    DeviceGuard g(r->device);
    if ((s = sync_pass(r)) != EDXR_OK)
        return s;
    bool textured = false;
    for (uint32_t v = 0; v < num_views; v++)
        textured = textured || views[v].ps_kind == EDXR_PS_LAMBERTIAN_TEXTURED;
    std::vector<edxr_mesh> dm(num_meshes);
    for (uint32_t m = 0; m < num_meshes; m++)
        if ((s = stage_mesh(r, m, &meshes[m], &dm[m], textured)) != EDXR_OK)
            return s;
    if ((s = ensure_frames_host(r, num_views)) != EDXR_OK)
        return s;
    cudaEventSynchronize(r->done);
    for (uint32_t v = 0; v < num_views; v++)
    {
        Camera cam;
        std::memcpy(cam.mv, views[v].mv, 64);
        std::memcpy(cam.proj, views[v].proj, 64);
        std::memcpy(cam.raster, views[v].raster, 64);
        cam.set = true;
        Shading sh;
        sh.ps_kind = views[v].ps_kind;
        sh.p = views[v].shading;
        fill_frame(r->frames_host[v], dm[views[v].mesh], cam, sh, views[v].depth_func, r->state.hierarchical, width,
                   height, r);
    }
    return launch_frames(r, num_views, width, height);
}

edxr_status edxr_get_batch_outputs(edxr_renderer* r, edxr_batch_outputs* out)
{
    if (!r || !out)
        return fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    DeviceGuard g(r->device);
    edxr_status s = sync_pass(r);
    if (s != EDXR_OK)
        return s;
    if (!r->last_frames)
        return fail(EDXR_ERR_INVALID_ARG, "nothing rendered yet");
    out->color = r->color.as<float>();
    out->depth = r->depth.as<float>();
    out->triangle_id = r->tri_id.as<uint32_t>();
    out->num_views = r->last_frames;
    out->width = r->out_width;
    out->height = r->out_height;
    return EDXR_OK;
}

edxr_status edxr_read_batch_outputs(edxr_renderer* r, uint32_t first_view, uint32_t num_views, float* color,
                                    float* depth, uint32_t* id)
{
    if (!r)
        return fail(EDXR_ERR_INVALID_ARG, "NULL renderer");
    DeviceGuard g(r->device);
    edxr_status s = sync_pass(r);
    if (s != EDXR_OK)
        return s;
    if (!r->last_frames || (uint64_t)first_view + num_views > r->last_frames)
        return fail(EDXR_ERR_INVALID_ARG, "view range outside the last pass");
    const size_t per = (size_t)r->out_width * r->out_height;
    const size_t off = per * first_view, n = per * num_views;
    if (color) EDXR_CUDA(cudaMemcpyAsync(color, r->color.as<float>() + 4 * off, 16 * n, cudaMemcpyDeviceToHost, r->stream));
    if (depth) EDXR_CUDA(cudaMemcpyAsync(depth, r->depth.as<float>() + off, 4 * n, cudaMemcpyDeviceToHost, r->stream));
    if (id) EDXR_CUDA(cudaMemcpyAsync(id, r->tri_id.as<uint32_t>() + off, 4 * n, cudaMemcpyDeviceToHost, r->stream));
    EDXR_CUDA(cudaStreamSynchronize(r->stream));
    return EDXR_OK;
}

namespace {

// The mesh of the differentiable form must be device-resident and have the
// vertex/triangle counts every frame of the last pass was rendered with.
edxr_status diff_mesh(edxr_renderer* r, const edxr_mesh* mesh, const edxr_shader_params* params, DiffMesh* m)
{
    edxr_status s = check_mesh(mesh);
    if (s != EDXR_OK)
        return s;
    std::memset(m, 0, sizeof(*m));
    if (params)
    {
        m->override_shading = 1;
        for (int q = 0; q < 3; q++)
            m->light[q] = params->light[q];
        m->ks = params->ks;
        m->shininess = params->shininess;
    }
    if (mesh->memory != EDXR_MEMORY_DEVICE)
        return fail(EDXR_ERR_INVALID_ARG, "the differentiable form takes a device-memory mesh");
    if ((s = sync_pass(r)) != EDXR_OK)
        return s;
    if (!r->last_frames)
        return fail(EDXR_ERR_INVALID_ARG, "nothing rendered yet");
    if (r->last_samples != 1)
        return fail(EDXR_ERR_UNSUPPORTED, "the differentiable form takes a pass rendered with one sample per pixel");
    for (uint32_t i = 0; i < r->last_frames; i++)
        if (r->frames_host[i].ps_kind == EDXR_PS_LAMBERTIAN_TEXTURED)
            return fail(EDXR_ERR_UNSUPPORTED, "the differentiable form has no adjoint of texture sampling");
    for (uint32_t i = 0; i < r->last_frames; i++)
        if (r->frames_host[i].nv != mesh->num_vertices || r->frames_host[i].nt != mesh->num_triangles)
            return fail(EDXR_ERR_INVALID_ARG, "mesh sizes differ from the mesh of the last pass");
    m->positions = static_cast<const char*>(mesh->positions);
    m->normals = static_cast<const char*>(mesh->normals);
    m->albedo = static_cast<const char*>(mesh->albedo);
    m->indices = mesh->indices;
    m->pos_stride = mesh->position_stride;
    m->nrm_stride = mesh->normal_stride;
    m->alb_stride = mesh->albedo_stride;
    m->nv = mesh->num_vertices;
    m->nt = mesh->num_triangles;
    return EDXR_OK;
}

}  // namespace

edxr_status edxr_shade_visible(edxr_renderer* r, const edxr_mesh* mesh, const edxr_shader_params* params,
                               float* color_out)
{
    if (!r || !color_out)
        return fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    DeviceGuard g(r->device);
    DiffMesh m;
    edxr_status s = diff_mesh(r, mesh, params, &m);
    if (s != EDXR_OK)
        return s;
    const uint64_t total = (uint64_t)r->last_frames * r->out_width * r->out_height;
    EDXR_CUDA(launch_shade_visible(r->last, total, m, reinterpret_cast<float4*>(color_out), r->stream));
    EDXR_CUDA(cudaStreamSynchronize(r->stream));
    return EDXR_OK;
}

edxr_status edxr_backward(edxr_renderer* r, const edxr_mesh* mesh, const edxr_shader_params* params,
                          const float* grad_color, const edxr_grads* grads)
{
    if (!r || !grad_color || !grads)
        return fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    DeviceGuard g(r->device);
    DiffMesh m;
    edxr_status s = diff_mesh(r, mesh, params, &m);
    if (s != EDXR_OK)
        return s;
    EDXR_CUDA(r->diff_scratch.ensure(8 * sizeof(double)));
    DiffGrads dg;
    dg.albedo = grads->albedo;
    dg.normals = grads->normals;
    dg.positions = grads->positions;
    dg.light = grads->light;
    dg.ks = grads->ks;
    dg.shininess = grads->shininess;
    dg.scratch = r->diff_scratch.as<double>();
    const uint64_t total = (uint64_t)r->last_frames * r->out_width * r->out_height;
    EDXR_CUDA(launch_backward(r->last, total, m, reinterpret_cast<const float4*>(grad_color), dg, r->stream));
    EDXR_CUDA(cudaEventRecord(r->done, r->stream));
    return EDXR_OK;
}

}  // extern "C"
