// edxr_render_noalloc: one frame of the pipeline for callers that cannot
// allocate device memory.
//
// Some hosts own every byte of device memory themselves — an engine or plugin
// host that hands the renderer a fixed budget, or a render loop that must not
// call cudaMalloc / cudaFree because those synchronise the whole device and
// stall other work in flight.  This entry point serves them: the caller passes
// the mesh (device memory), the camera and the output images (device memory),
// and every intermediate buffer of the pass — clip positions, set-up
// triangles, clipped polygons, per-tile counters and bins, the status word —
// lives in one file-scope __device__ array of fixed size.  Nothing here calls
// cudaMalloc, cudaFree or any allocating routine.
//
// Rules for callers:
//  * The array is part of the library image: every GPU that loads the library
//    holds kNoAllocScratchBytes of it until the process exits.
//  * The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current).
//  * Every call on a device shares the one array and leaves its contents
//    behind; the pass clears what must start at zero itself.  Calls whose GPU
//    work overlaps (several host threads, or several streams) race on the
//    array: serialise them.
//  * Sizes beyond the fixed limits below are rejected with
//    EDXR_ERR_INVALID_ARG before any GPU work; a frame whose bins do not fit
//    fails with EDXR_ERR_OVERFLOW (nothing can grow).
//  * Every call blocks the calling thread: it copies the frame descriptor
//    from its own stack, then waits on `stream` for the frame and reads the
//    status word back before returning.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "edxr.h"
#include "edxr_internal.h"

using namespace edxr;

namespace {

constexpr uint32_t kMaxVertices = 65536;
constexpr uint32_t kMaxTriangles = 65536;
constexpr uint32_t kMaxSide = 4096;
constexpr uint32_t kMaxPixels = 1u << 20;
constexpr uint32_t kMaxTiles = 4608;  // >= ceil(W/16)*ceil(H/16) for W*H <= 2^20, W,H <= 4096
constexpr uint32_t kRtriCap = kMaxTriangles + kMaxTriangles / 4;
constexpr uint32_t kPolyCap = 8192;
constexpr uint32_t kBigCap = kRtriCap;
constexpr uint32_t kBinCap = 3u << 18;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// byte offsets of the sub-buffers inside the array
constexpr size_t kOffFrame = 0;
constexpr size_t kOffRtri = align256(kOffFrame + sizeof(FrameDesc));
constexpr size_t kOffRtriZlo = kOffRtri + sizeof(RTri) * (size_t)kRtriCap;
constexpr size_t kOffPoly = align256(kOffRtriZlo + 4 * (size_t)kRtriCap);
constexpr size_t kOffClipList = align256(kOffPoly + sizeof(ClipPoly) * (size_t)kPolyCap);
constexpr size_t kOffCount = align256(kOffClipList + 4 * (size_t)kPolyCap);
constexpr size_t kOffOffset = align256(kOffCount + 4 * (size_t)(kMaxTiles + 1));
constexpr size_t kOffCursor = align256(kOffOffset + 4 * (size_t)(kMaxTiles + 1));
constexpr size_t kOffZocc = align256(kOffCursor + 4 * (size_t)(kMaxTiles + 1));
constexpr size_t kOffBins = align256(kOffZocc + 4 * (size_t)(kMaxTiles + 1));
constexpr size_t kOffBinTmp = align256(kOffBins + 4 * (size_t)kBinCap);
constexpr size_t kOffBig = align256(kOffBinTmp + 8 * (size_t)kBinCap);
constexpr size_t kOffCounters = align256(kOffBig + 4 * (size_t)kBigCap);
constexpr size_t kOffStatus = align256(kOffCounters + 4 * kCounters + 8 * (size_t)scan_blocks(kMaxTiles));
constexpr size_t kOffTriFirst = align256(kOffStatus + sizeof(DeviceStatus));
constexpr size_t kItemCap = item_capacity(kMaxTiles, kBinCap);
constexpr size_t kOffItems = align256(kOffTriFirst + 4 * (size_t)kMaxTriangles);
constexpr size_t kOffKeyBuf = align256(kOffItems + sizeof(uint4) * kItemCap);
constexpr size_t kNoAllocScratchBytes = align256(kOffKeyBuf + 8 * (size_t)kMaxPixels);

// The scratch of edxr_render_noalloc (about 24 MiB per device).  Host code
// only ever sees a host-side stand-in for this name; its device address comes
// from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};
int g_sms[kMaxDevices] = {};

// Messages go to edxr_last_error_string like every other entry point.
edxr_status noalloc_fail(edxr_status s, const char* msg)
{
    record_error(msg);
    return s;
}

// Per-device set-up, with `device` current: the array's device address and
// the SM count used to size the persistent grids.
edxr_status scratch_for_device(int device, unsigned char** base, int* sms)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[device])
    {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return noalloc_fail(EDXR_ERR_CUDA, "cudaGetSymbolAddress of the no-alloc scratch failed");
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device);
        if (e != cudaSuccess)
            return noalloc_fail(EDXR_ERR_CUDA, "cudaDeviceGetAttribute failed");
        prepare_kernels();
        g_sms[device] = n;
        g_scratch_ptr[device] = ptr;
    }
    *base = static_cast<unsigned char*>(g_scratch_ptr[device]);
    *sms = g_sms[device];
    return EDXR_OK;
}

}  // namespace

extern "C" {

edxr_status edxr_render_noalloc(const edxr_mesh* mesh, const float mv[16], const float proj[16],
                                const float raster[16], const edxr_state* state, int ps_kind,
                                const edxr_shader_params* params, uint32_t width, uint32_t height,
                                float* color, float* depth, uint32_t* triangle_id, void* stream)
{
    if (!mesh || !mv || !proj || !raster || !state || !params || !color || !depth || !triangle_id)
        return noalloc_fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    if (mesh->memory != EDXR_MEMORY_DEVICE)
        return noalloc_fail(EDXR_ERR_INVALID_ARG, "the mesh must be in device memory (nothing can be staged)");
    if (mesh->num_triangles > 0 && (!mesh->positions || !mesh->indices))
        return noalloc_fail(EDXR_ERR_INVALID_ARG, "mesh positions and indices are required");
    if (mesh->positions && mesh->position_stride < 12)
        return noalloc_fail(EDXR_ERR_INVALID_ARG, "position stride below 12 bytes");
    if ((mesh->normals && mesh->normal_stride < 12) || (mesh->albedo && mesh->albedo_stride < 12))
        return noalloc_fail(EDXR_ERR_INVALID_ARG, "attribute stride below 12 bytes");
    if (mesh->num_vertices > kMaxVertices)
        return noalloc_fail(EDXR_ERR_INVALID_ARG, "more than 65536 vertices: over the fixed no-alloc scratch limit");
    if (mesh->num_triangles > kMaxTriangles)
        return noalloc_fail(EDXR_ERR_INVALID_ARG, "more than 65536 triangles: over the fixed no-alloc scratch limit");
    if (width == 0 || height == 0 || width > kMaxSide || height > kMaxSide ||
        (uint64_t)width * height > kMaxPixels)
        return noalloc_fail(EDXR_ERR_INVALID_ARG,
                            "framebuffer must be at most 4096 on a side and 2^20 pixels: fixed no-alloc scratch limit");
    if (state->depth_func != EDXR_DEPTH_LEQUAL && state->depth_func != EDXR_DEPTH_LESS)
        return noalloc_fail(EDXR_ERR_INVALID_ARG, "unknown depth function");
    if (state->msaa_log2 != 0)
        return noalloc_fail(EDXR_ERR_UNSUPPORTED, "edxr_render_noalloc renders one sample per pixel (msaa_log2 must be 0)");
    if (ps_kind == EDXR_PS_LAMBERTIAN_TEXTURED)
        return noalloc_fail(EDXR_ERR_UNSUPPORTED, "edxr_render_noalloc holds no texture slots");
    if (ps_kind < EDXR_PS_BLINN_PHONG || ps_kind > EDXR_PS_LAMBERTIAN)
        return noalloc_fail(EDXR_ERR_INVALID_ARG, "unknown pixel shader");
    const double ln = sqrt((double)params->light[0] * params->light[0] + (double)params->light[1] * params->light[1] +
                           (double)params->light[2] * params->light[2]);
    if (!(ln > 0.0) || !isfinite(ln))
        return noalloc_fail(EDXR_ERR_INVALID_ARG, "light direction must be a finite non-zero vector");

    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices)
        return noalloc_fail(EDXR_ERR_CUDA, "no current CUDA device");
    unsigned char* base = nullptr;
    int sms = 0;
    edxr_status st = scratch_for_device(device, &base, &sms);
    if (st != EDXR_OK)
        return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    FrameDesc f;
    memset(&f, 0, sizeof(f));
    frame_mesh(f, *mesh, width, height);
    f.depth_func = state->depth_func;
    f.hierarchical = state->hierarchical ? 1 : 0;
    frame_camera(f, mv, proj, raster);
    frame_shading(f, ps_kind, params->light, params->ks, params->shininess);
    const uint32_t tiles = (uint32_t)(f.tdx * f.tdy);

    PassArgs a;
    memset(&a, 0, sizeof(a));
    a.tune = default_tuning();
    a.frames = reinterpret_cast<const FrameDesc*>(base + kOffFrame);
    a.num_frames = 1;
    a.tiles_per_frame = 0;  // (one frame: the search is one step)
    a.total_vertices = f.nv;
    a.total_tris = f.nt;
    a.total_tiles = tiles;
    a.rtris = reinterpret_cast<RTri*>(base + kOffRtri);
    a.rtri_zlo = reinterpret_cast<uint32_t*>(base + kOffRtriZlo);
    a.rtri_capacity = kRtriCap;
    a.polys = reinterpret_cast<ClipPoly*>(base + kOffPoly);
    a.clip_list = reinterpret_cast<uint32_t*>(base + kOffClipList);
    a.poly_capacity = kPolyCap;
    a.tile_count = reinterpret_cast<uint32_t*>(base + kOffCount);
    a.tile_offset = reinterpret_cast<uint32_t*>(base + kOffOffset);
    a.tile_cursor = reinterpret_cast<uint32_t*>(base + kOffCursor);
    a.tile_zocc = reinterpret_cast<uint32_t*>(base + kOffZocc);
    a.bins = reinterpret_cast<uint32_t*>(base + kOffBins);
    a.bin_tmp = reinterpret_cast<uint2*>(base + kOffBinTmp);
    a.bin_capacity = kBinCap;
    a.big_list = reinterpret_cast<uint32_t*>(base + kOffBig);
    a.big_capacity = kBigCap;
    a.counters = reinterpret_cast<uint32_t*>(base + kOffCounters);
    a.scan_status = reinterpret_cast<unsigned long long*>(a.counters + kCounters);
    a.status = reinterpret_cast<DeviceStatus*>(base + kOffStatus);
    a.color = reinterpret_cast<float4*>(color);
    a.depth = depth;
    a.tri_id = triangle_id;
    a.tri_first = reinterpret_cast<uint32_t*>(base + kOffTriFirst);
    a.items = reinterpret_cast<uint4*>(base + kOffItems);
    a.item_capacity = kItemCap;
    // zero in the array's initial image, and every pass leaves it zero
    a.keybuf = reinterpret_cast<unsigned long long*>(base + kOffKeyBuf);
    a.total_pixels = (uint64_t)width * height;
    a.num_sms = sms;

    // The descriptor travels from this stack frame; a pageable source makes
    // the copy complete before cudaMemcpyAsync returns.
    if (cudaMemcpyAsync(base + kOffFrame, &f, sizeof(f), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return noalloc_fail(EDXR_ERR_CUDA, "descriptor upload failed");
    if (launch_pipeline(a, s) != cudaSuccess)
        return noalloc_fail(EDXR_ERR_CUDA, "kernel launch failed");
    DeviceStatus ds;
    if (cudaMemcpyAsync(&ds, base + kOffStatus, sizeof(ds), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return noalloc_fail(EDXR_ERR_CUDA, "frame execution failed");
    if (ds.error)
        return noalloc_fail((edxr_status)ds.error, ds.error == EDXR_ERR_INVALID_ARG
                                                       ? "a triangle references a vertex index out of range"
                                                       : "the device reported an error (a bounded wait ran out)");
    if (ds.overflow)
        return noalloc_fail(EDXR_ERR_OVERFLOW, "the frame needs more bins or clipped polygons than the fixed scratch holds");
    return EDXR_OK;
}

}  // extern "C"
