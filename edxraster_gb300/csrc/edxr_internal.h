// Internal definitions shared by the host code and the CUDA kernels of the
// EDXRaster GB300 pipeline.  Everything here is a layout in device memory.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "edxr.h"

namespace edxr {

// 16x16-pixel bin tiles.  Each is exactly one quadrant of a 32x32 tile of the
// reference (Tile::SIZE_LOG_2 = 5, Tile.h:12), so the reference's per-32-tile
// and per-quadrant decisions (Renderer.cpp:173-227, Rasterizer.h:32-111) map
// onto a 16x16 tile without change.
constexpr int kTileLog2 = 4;
constexpr int kTileSize = 1 << kTileLog2;
constexpr int kRefTileLog2 = 5;

// Decision of the reference for one (triangle, 16x16 tile) pair.
constexpr uint32_t kDecisionAccept = 1;  // every pixel is depth-tested, no edge test
constexpr uint32_t kDecisionFine = 2;    // pixel edge test inside the bounding box

constexpr uint32_t kUnclipped = 0xFFFFFFFFu;
constexpr uint32_t kNoTriangle = 0xFFFFFFFFu;
// Raster work item: up to this many bin entries of one tile.  A tile with
// more entries is split into several items whose winners are merged in a
// per-pixel key buffer before the last of them shades the tile.
constexpr uint32_t kItemEntries = 128;  // default bin entries per raster work item (Tuning::item_entries)
// Tile-count scan: tiles per block, and blocks (one status word each) of a pass.
constexpr int kScanItems = 4;
constexpr int kScanThreads = 256;
constexpr int kScanBlock = kScanItems * kScanThreads;
__host__ __device__ constexpr uint32_t scan_blocks(uint64_t tiles)
{
    return (uint32_t)((tiles + kScanBlock - 1) / kScanBlock);
}
// The unsorted bin list is kBinStripes regions of bin_capacity / kBinStripes
// slots, each filled through its own counter (one 128-byte line apart, from
// word kStripeBase of PassArgs::counters): word 0 the region's used slots,
// word 1 the unclipped triangles that survived setup in warps of that
// stripe (statistics).  Warps append to stripe (warp index mod kBinStripes),
// so no block-wide barrier is needed to keep one counter from being the
// single address every warp of the grid contends for.
constexpr int kBinStripes = 32;
constexpr int kStripeStride = 32;
constexpr int kStripeBase = 16;
constexpr int kCounters = kStripeBase + kBinStripes * kStripeStride;  // words of PassArgs::counters
__host__ __device__ constexpr uint64_t stripe_slots(uint64_t bin_capacity) { return bin_capacity / kBinStripes; }
// Work items of a pass: one per tile plus one per item_entries bin entries.
constexpr uint64_t item_capacity(uint64_t tiles, uint64_t bin_capacity, uint32_t item_entries = kItemEntries)
{
    return tiles + bin_capacity / item_entries + 1;
}
// 3 + one vertex per clip plane is 9 in exact arithmetic; rounding on nearly
// collinear vertices can add a few more, so the working polygon has room.
constexpr int kMaxPolygon = 16;

// One texture slot in device memory: level l (of `levels`, each half the
// size of the one before, down to 1x1) starts at texel base + sum of the
// sizes of the levels before it.
struct TexDesc
{
    uint32_t width, height, levels, pad;
    uint64_t base;
};

// Per frame (one view of one mesh).  Kernels read it from global memory.
struct FrameDesc
{
    // mesh (device pointers; strides in bytes)
    const char* positions; const char* normals; const char* albedo; const char* uvs;
    const uint32_t* indices;
    uint32_t pos_stride, nrm_stride, alb_stride, uv_stride;
    uint32_t nv, nt;
    // flattened work offsets of this frame
    uint32_t vtx_base;   // into the clip-position buffer
    uint32_t tri_base;   // into the flattened input-triangle space
    uint32_t tile_base;  // into the flattened 16x16-tile space
    uint32_t pad0;
    uint64_t pix_base;   // into the output images
    int width, height;
    int tdx, tdy;        // 16x16 tile grid
    int tdx32, tdy32;    // reference 32x32 tile grid
    int ps_kind, depth_func, hierarchical, pad1;
    float mvp[16];
    float raster[16];
    float eye[3];        // object-space eye position (MV^-1 * 0)
    float light[3];      // normalised light direction
    float ks, shininess;
    float ndc_from_raster[6];  // 2D affine inverse of the raster matrix (x, y rows)
    float light_raw[3];        // light direction as given (FP64 shading normalises it)
    float pad2;
    double eye_d[3];           // eye position in double (FP64 shading)
    double ndc_from_raster_d[6];  // the raster-to-NDC inverse in double (differentiable form)
    float ndc_from_raster_lo[6];  // ndc_from_raster_d - ndc_from_raster: with it, a float pair (hi + lo)
    float pad3[2];
    // textures of the textured Lambertian shader
    const uint32_t* tex_ids;      // per input triangle (NULL: slot 0)
    const TexDesc* textures;
    const float4* texels;
    uint32_t num_textures;
    int tex_filter;               // edxr_texture_filter
};

// One triangle after clipping and setup (RasterTriangle, RasterTriangle.h:11-24),
// 64 bytes, written by the setup kernel in any order; `order` restores the
// reference's submission order: input triangle * 16 + fan index.
struct __align__(16) RTri
{
    int v0x, v0y, v1x, v1y;
    int v2x, v2y;
    uint32_t order;
    uint32_t meta;       // bits 0-11: reject/accept corners (2 bits each), 12-31: frame index
    float invDet, z0, z1, z2;   // z after the post-pass (z_clip * (1/w))
    float invW0, invW1, invW2;
    uint32_t poly;       // kUnclipped, or (clipped-polygon index << 4) | fan index
};
static_assert(sizeof(RTri) == 64, "RTri must stay 64 bytes");

// Clip weights of the vertices of one clipped polygon (Clipper.h:123-152),
// relative to the source triangle's three vertices.
struct __align__(16) ClipPoly
{
    float w[kMaxPolygon][3];
    uint32_t n;
};

// Device status word, read back after every frame.
struct DeviceStatus
{
    uint32_t overflow;       // bins needed more than the capacity
    uint32_t error;          // EDXR_ERR_TIMEOUT and similar
    uint64_t bins_needed;    // bin-list capacity this frame needs (padded bins; the fullest stripe x stripes)
    uint32_t raster_tris;    // needed (may exceed the capacity)
    uint32_t clipped_polys;  // needed
    uint32_t big_tris;       // needed
    uint32_t rtri_slots;     // raster-triangle slots needed: input triangles + fan pieces
    uint64_t bin_entries;    // (triangle, tile) entries binned this frame
};

// Tunables of one pass (edxr_set_tuning; chosen by the autotuner).
struct Tuning
{
    int small_region;     // bin entries whose pixel region is at most this are rasterized triangle-parallel
    int raster_variant;   // 0/1: k_raster with the triangle-parallel path (3 / 5 blocks per SM), 2: pixel-parallel only
    int bin_blocks_per_sm;
    int raster_blocks_per_sm;  // 0 = as many as fit
    int item_entries;     // bin entries per raster work item; items of at least 3/4 of it are handed out first
    // Failure test of the scan's bounded wait (edxr_debug_scan_stall): scan
    // block scan_stall_block (-1: none) does not publish its sum, and a wait
    // gives up after scan_spin_limit polls (0: kScanSpinLimit).
    int scan_stall_block;
    int scan_spin_limit;
};

// Launch parameters shared by every kernel of one pass.
struct PassArgs
{
    Tuning tune;
    const FrameDesc* frames;
    uint32_t num_frames;
    uint32_t tiles_per_frame;  // every frame's tile count when they are equal (then frame = tile / it), else 0
    uint32_t* frame_of_block;  // several frames: the frame of triangle 256 b, per b (filled by k_clear); else NULL
    uint32_t total_vertices;
    int4* vrecs;             // per flattened vertex: setup record (vertex stage), or NULL: setup projects in place
    uint32_t total_tris;
    uint32_t total_tiles;
    RTri* rtris;             // slot i < total_tris: unclipped input triangle i; then fan pieces (counters[0])
    uint32_t* rtri_zlo;      // per raster-triangle slot: the lower bound of its depth keys (zmin_key)
    uint32_t rtri_capacity;
    ClipPoly* polys;
    uint32_t poly_capacity;  // also the capacity of clip_list
    uint32_t* clip_list;     // input triangles (flattened) that straddle a clip plane
    uint32_t* tile_count;    // total_tiles + 1; counts until the scan, then (zeroed by it) the entries of a split
                             // tile its items have rastered
    uint32_t* tile_offset;   // total_tiles + 1 (exclusive scan of padded counts)
    uint32_t* tile_zocc;     // total_tiles + 1; per tile the least far-depth key of the triangles accepted
                             // over it whole (entries beyond it are hidden), ~0 for none
    uint32_t* tile_cursor;   // total_tiles + 1; the scatter's cursors: after it, the entries each bin holds
    uint32_t* bins;
    uint2* bin_tmp;          // decided (tile, entry) pairs before the scatter, bin_capacity of them
    uint64_t bin_capacity;
    uint32_t* big_list;      // raster triangles with many tiles, binned by whole blocks
    uint32_t big_capacity;
    uint32_t* counters;      // [0] fan-piece slots, [2] big tris, [3] raster work queue, [4] clip list,
                             // [6] heavy raster work items, [7] light ones, [8] scan block tickets,
                             // [11] surviving fan pieces, [kStripeBase + r * kStripeStride] stripe r of the
                             // unsorted bin list (kCounters words)
    unsigned long long* scan_status;  // per scan block (scan_blocks(total_tiles) words)
    uint4* items;            // raster work items (tile | split flag, first entry, end entry, 0), one per
                             // item_entries-entry slice: heavy ones from the front, light ones from the back
    uint64_t item_capacity;
    unsigned long long* keybuf;  // per pixel: ~(smallest key) of split tiles, 0 between passes
    DeviceStatus* status;
    uint32_t* tri_first;     // per clipped input triangle: its first fan piece
    float4* color;
    float* depth;
    uint32_t* tri_id;        // the winner's input-triangle id (kNoTriangle: background)
    uint64_t total_pixels;   // frames * width * height
    int msaa_log2;           // samples per pixel = 1 << msaa_log2; depth and tri_id hold one plane per sample
    int num_sms;
};

constexpr int kMaxMsaaLog2 = 5;  // 32 samples (CoverageMask, Shader.h:52-54)

// Host-side launchers (edxr_kernels.cu).
constexpr int kStageEvents = 6;  // boundaries of the 5 timed stages
// ev: NULL, or kStageEvents events recorded around the stages.
cudaError_t launch_pipeline(const PassArgs& a, cudaStream_t s, cudaEvent_t* ev = nullptr);
int kernels_per_pass(const PassArgs& a);
Tuning default_tuning();
// Sets the message edxr_last_error_string returns on this thread.
void record_error(const char* msg);
void prepare_kernels();
// Host-side fill of a frame descriptor, shared by every entry point so that
// all of them hand the kernels identical frames (edxr_api.cu).
// C = A * B of row-major 4x4 matrices, each entry summed left to right in float.
void mat_mul(const float* A, const float* B, float* C);
// Object-space eye position MV^-1 * 0 in double; false if MV is singular.
bool eye_from_mv(const float* mv, double eye[3]);
// Mesh pointers, strides, counts and the framebuffer's tile grids.
void frame_mesh(FrameDesc& f, const edxr_mesh& m, uint32_t width, uint32_t height);
// MVP = proj * mv, the raster matrix, the eye position and the raster-to-NDC inverse.
void frame_camera(FrameDesc& f, const float mv[16], const float proj[16], const float raster[16]);
// Pixel shader kind, normalised and raw light direction, ks and shininess.
void frame_shading(FrameDesc& f, int ps_kind, const float light[3], float ks, float shininess);
cudaError_t launch_back_buffer(const float4* color, uint8_t* rgba8, int width, int height, cudaStream_t s);
// One mip level: each texel the mean of the 2x2 texels above it (indices
// clamped to the source size).
cudaError_t launch_mip_level(const float4* src, int sw, int sh, float4* dst, int dw, int dh, cudaStream_t s);
// Mesh used by the differentiable form (device pointers, strides in bytes).
struct DiffMesh
{
    const char* positions; const char* normals; const char* albedo;
    const uint32_t* indices;
    uint32_t pos_stride, nrm_stride, alb_stride;
    uint32_t nv, nt;
    int override_shading;   // 1: use light/ks/shininess below for every frame
    float light[3], ks, shininess;
};
struct DiffGrads
{
    float* albedo; float* normals; float* positions;  // nv*3 each, may be NULL
    float* light; float* ks; float* shininess;         // may be NULL
    double* scratch;                                    // 5 doubles, zeroed by the launcher
};
cudaError_t launch_shade_visible(const PassArgs& a, uint64_t total_pixels, const DiffMesh& m, float4* out,
                                 cudaStream_t s);
cudaError_t launch_backward(const PassArgs& a, uint64_t total_pixels, const DiffMesh& m, const float4* grad,
                            const DiffGrads& g, cudaStream_t s);

}  // namespace edxr
