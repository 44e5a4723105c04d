/*
 * edxr.h — C ABI of the GB300-native EDXRaster rasterization pipeline.
 *
 * This is the drop-in boundary for EDXRaster's Renderer (EDXRaster/Core/
 * Renderer.h:15-59): the same per-frame pipeline — vertex transform,
 * homogeneous clipping, 1/16-pixel fixed-point setup, binning, hierarchical
 * edge-function rasterization, perspective-correct interpolation, shading and
 * the depth test — runs as CUDA kernels for sm_103a behind plain C entry
 * points.  Signatures carry only plain pointers, sizes and POD structs.
 *
 * Semantics kept from the reference:
 *   - triangle coverage, the depth value and the winning triangle of every
 *     pixel are bit-identical to Renderer::RenderMesh (Renderer.cpp:100-118)
 *     on the same inputs, including its top-left rule, int32 wraparound,
 *     back-face culling (det <= 0, RasterTriangle.h:49-51) and
 *     submission-order tie breaking under LEQUAL (FrameBuffer.cpp:64);
 *   - matrices are the reference's three (SetTransform, Renderer.cpp:85-92):
 *     model-view, projection and the NDC->raster matrix, row-major with
 *     column vectors (p' = M * p).
 * Differences:
 *   - outputs are linear, top-down RGBA32F colour, D32F depth and a u32
 *     triangle-id buffer on the device (the reference keeps bottom-up RGBA8 and
 *     a tiled depth buffer, FrameBuffer.cpp:39-42,54-68); edxr_get_back_buffer
 *     gives the reference's bottom-up RGBA8 view;
 *   - errors are reported as edxr_status instead of being ignored;
 *   - several renderers may live in one process (the reference keeps a
 *     process-wide RenderStates singleton, RenderStates.h:38-44); one renderer
 *     must be used from one host thread at a time.
 *
 * Asynchrony: edxr_render* and edxr_backward enqueue work on the renderer's
 * stream and return.  edxr_synchronize / edxr_get_outputs / edxr_read_outputs
 * wait for the frame, check the device status word and, when a bin buffer
 * overflowed, grow it and render the frame again before returning.
 */
#ifndef EDXR_H
#define EDXR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EDXR_ABI_VERSION 1

typedef enum edxr_status
{
    EDXR_OK = 0,
    EDXR_ERR_INVALID_ARG = 1,  /* bad pointer, size, enum or index          */
    EDXR_ERR_OVERFLOW = 2,     /* a capacity limit could not be met          */
    EDXR_ERR_TIMEOUT = 3,      /* a device wait gave up (work queue)         */
    EDXR_ERR_CUDA = 4,         /* a CUDA runtime call failed                 */
    EDXR_ERR_OUT_OF_MEMORY = 5,
    EDXR_ERR_UNSUPPORTED = 6   /* valid request this build does not provide  */
} edxr_status;

typedef struct edxr_renderer edxr_renderer;

typedef enum edxr_memory
{
    EDXR_MEMORY_HOST = 0,   /* pointers are host memory, read per call (see edxr_mesh) */
    EDXR_MEMORY_DEVICE = 1  /* pointers are device memory of the renderer GPU */
} edxr_memory;

typedef enum edxr_depth_func
{
    EDXR_DEPTH_LEQUAL = 0,  /* reference behaviour (FrameBuffer.cpp:64)  */
    EDXR_DEPTH_LESS = 1
} edxr_depth_func;

typedef enum edxr_vs_kind
{
    EDXR_VS_DEFAULT = 0     /* DefaultVertexShader, Shader.h:37-50 */
} edxr_vs_kind;

typedef enum edxr_ps_kind
{
    /* albedo*(max(N.L,0)+0.2)*3/pi + ks*max(N.H,0)^shininess, per-vertex albedo */
    EDXR_PS_BLINN_PHONG = 0,
    /* BlinnPhongPixelShader as written (Shader.h:246-282): no albedo, no clamp
     * on N.H; the reference constants are ks = 3, shininess = 200            */
    EDXR_PS_BLINN_PHONG_REFERENCE = 1,
    /* LambertianAlbedoPixelShader (Shader.h:209-244) with per-vertex albedo in
     * place of the texture lookup                                             */
    EDXR_PS_LAMBERTIAN_ALBEDO = 2,
    /* LambertianPixelShader (Shader.h:185-207)                                */
    EDXR_PS_LAMBERTIAN = 3,
    /* LambertianAlbedoPixelShader as written (Shader.h:209-244): the albedo is
     * sampled from the triangle's texture (edxr_set_textures, the mesh's
     * per-triangle texture ids) with the state's texture filter; the mesh
     * needs texture coordinates                                              */
    EDXR_PS_LAMBERTIAN_TEXTURED = 4
} edxr_ps_kind;

/* Texture filters (TextureFilter of RenderStates::TexFilter, RenderStates.h:23;
 * the reference's default is trilinear, RenderStates.h:60). */
typedef enum edxr_texture_filter
{
    EDXR_FILTER_NEAREST = 0,
    EDXR_FILTER_LINEAR = 1,
    EDXR_FILTER_TRILINEAR = 2,
    EDXR_FILTER_ANISOTROPIC_4X = 3,
    EDXR_FILTER_ANISOTROPIC_8X = 4,
    EDXR_FILTER_ANISOTROPIC_16X = 5
} edxr_texture_filter;

typedef enum edxr_texture_format
{
    EDXR_TEXTURE_RGBA8 = 0,    /* 4 bytes per texel, channel = byte / 255      */
    EDXR_TEXTURE_RGBA32F = 1   /* 16 bytes per texel                           */
} edxr_texture_format;

/* One texture (Texture2D<Color> of Mesh::mTextures, Mesh.h:25): texels in rows
 * of `width`, row 0 at v = 0; coordinates repeat.  A 1x1 texture is the
 * reference's ConstantTexture2D. */
typedef struct edxr_texture
{
    uint32_t width, height;
    int format;                /* edxr_texture_format                          */
    const void* texels;        /* host memory, copied by edxr_set_textures     */
} edxr_texture;

typedef struct edxr_init
{
    uint32_t width, height;  /* framebuffer size (Renderer::Initialize)     */
    void* stream;            /* cudaStream_t to enqueue on; NULL = legacy   */
    int device;              /* CUDA device ordinal                         */
} edxr_init;

typedef struct edxr_state
{
    int depth_func;          /* edxr_depth_func                              */
    int hierarchical;        /* RenderStates::HierarchicalRasterize (1)      */
    int msaa_log2;           /* RenderStates::MultiSampleLevel: 0..5 = 1..32 samples */
    int texture_filter;      /* RenderStates::TexFilter: edxr_texture_filter  */
} edxr_state;

typedef struct edxr_shader_params
{
    float light[3];          /* direction towards the light, object space; normalised inside */
    float ks;                /* specular weight                                             */
    float shininess;         /* specular exponent                                           */
} edxr_shader_params;

/* One indexed triangle mesh (Mesh.h:17-69 / InputBuffer.h:16-205).  Strides
 * are in bytes; positions, normals and albedo are three floats, uvs two.
 * The reference's interleaved Vertex_PositionNormalTex (32 bytes: position
 * at 0, normal at 12, uv at 24) is positions=base, normals=base+12,
 * uvs=base+24 with all strides 32.
 * With EDXR_MEMORY_HOST, positions and indices are copied to the device by
 * every render call; normals, albedo, uvs and texture ids are copied too,
 * unless they are page-locked (cudaHostAlloc, cudaHostRegister): the
 * shading then reads them in place, and only the winning triangles'
 * vertices cross the host link.  Host arrays stay unchanged until the frame
 * completes (edxr_synchronize). */
typedef struct edxr_mesh
{
    const void* positions; uint32_t position_stride;
    const void* normals;   uint32_t normal_stride;   /* NULL: (0,0,0)  */
    const void* uvs;       uint32_t uv_stride;       /* NULL: (0,0)    */
    const void* albedo;    uint32_t albedo_stride;   /* NULL: (1,1,1)  */
    const uint32_t* indices;                         /* 3 per triangle */
    uint32_t num_vertices;
    uint32_t num_triangles;
    int memory;                                      /* edxr_memory    */
    /* per-triangle texture slot (Mesh::mTexIdx, Mesh.h:26; Clipper.h:95), in
     * the same memory as the other arrays; NULL: slot 0 for every triangle */
    const uint32_t* texture_ids;
} edxr_mesh;

/* Renderer-owned device buffers, valid until the next render or resize.
 * With S = 2^msaa_log2 samples per pixel, depth and triangle_id hold S
 * planes of width*height (sample s at offset s*width*height) and colour is
 * the reference's resolve (FrameBuffer::Resolve, FrameBuffer.cpp:70-87): the
 * samples' 8-bit colours (each shaded at the pixel centre) averaged in
 * float, alpha = covered samples / S. */
typedef struct edxr_outputs
{
    float* color;            /* width*height*4 RGBA32F, row 0 = top; alpha 1 where covered */
    float* depth;            /* S*width*height D32F, cleared to 1.0                        */
    uint32_t* triangle_id;   /* S*width*height input-triangle index, 0xFFFFFFFF = none      */
    uint32_t width, height;
    uint32_t samples;        /* S                                                          */
} edxr_outputs;

typedef struct edxr_stats
{
    uint64_t raster_triangles;  /* triangles that survived clipping and culling */
    uint64_t bin_entries;       /* (triangle, 16x16 tile) pairs                   */
    uint64_t bin_capacity;
    uint32_t rerenders;         /* frames re-run after a bin overflow             */
    uint32_t tile_size;
    uint32_t kernels_per_pass;  /* CUDA kernels one render pass launches          */
    uint32_t clipped_polygons;  /* input triangles split by the clipper           */
} edxr_stats;

/* ---- lifetime (Renderer::Initialize / ~Renderer, Renderer.cpp:22-62,365-371) */
edxr_status edxr_create(edxr_renderer** out, const edxr_init* init);
edxr_status edxr_destroy(edxr_renderer* r);

/* Renderer::Resize, Renderer.cpp:64-83. */
edxr_status edxr_resize(edxr_renderer* r, uint32_t width, uint32_t height);

/* Renderer::SetTransform, Renderer.cpp:85-92.  Each matrix is 16 floats. */
edxr_status edxr_set_transform(edxr_renderer* r, const float mv[16], const float proj[16],
                               const float raster[16]);

/* RenderStates fields (RenderStates.h:15-28) and the setters of Renderer.h:47-49
 * (SetMSAAMode, SetTextureFilter, SetHierarchicalRasterize).  With
 * msaa_log2 > 0 (Renderer::SetMSAAMode, Renderer.cpp:94-98) edxr_render
 * rasterizes 2^msaa_log2 samples per pixel (FineRasterize_MultiSample /
 * TrivialAcceptTriangle_MultiSample, Rasterizer.h:202-300, 355-415); the
 * batched and differentiable forms and edxr_render_noalloc take one sample
 * per pixel and return EDXR_ERR_UNSUPPORTED otherwise. */
edxr_status edxr_set_state(edxr_renderer* r, const edxr_state* state);

/* Shader selection (the reference hard-wires it in Renderer::Initialize,
 * Renderer.cpp:40-41).  params may be NULL for the defaults. */
edxr_status edxr_set_shader(edxr_renderer* r, int vs_kind, int ps_kind,
                            const edxr_shader_params* params);

/* The texture slots (RenderStates::TextureSlots, RenderStates.h:28, filled
 * from Mesh::GetTextures in RenderMesh, Renderer.cpp:106): copies the texels
 * and builds each texture's mip chain on the device (box filter).  Replaces
 * the previous set; count 0 clears it. */
edxr_status edxr_set_textures(edxr_renderer* r, const edxr_texture* textures, uint32_t count);

/* ------------------------------------------------------------------------
 * Mesh input (Mesh::LoadMesh, Mesh.cpp:11-34, over EDXUtil's ObjMesh, which
 * the reference does not include): a Wavefront OBJ file with its MTL
 * materials, loaded into host arrays ready for edxr_mesh and
 * edxr_set_textures.  Faces are fanned into triangles; every distinct
 * (position, texture coordinate, normal) corner becomes one vertex; missing
 * normals are the area-weighted mean of the adjacent face normals.  The
 * transform is scale, then rotation about x, y, z (degrees, in that order),
 * then translation, as LoadMesh(pos, scl, rot, path) takes them.  Each
 * material is one texture slot: its map_Kd image (binary PPM or uncompressed
 * 24/32-bit BMP) or a 1x1 texture of its Kd colour; a triangle's texture id
 * is the slot of its usemtl material (slot 0, white, when there is none). */
typedef struct edxr_obj_mesh
{
    uint32_t num_vertices, num_triangles, num_textures;
    float* positions;          /* num_vertices x 3                                */
    float* normals;            /* num_vertices x 3                                */
    float* uvs;                /* num_vertices x 2                                */
    uint32_t* indices;         /* num_triangles x 3                               */
    uint32_t* texture_ids;     /* num_triangles                                   */
    edxr_texture* textures;    /* num_textures, RGBA32F texels owned by the mesh  */
} edxr_obj_mesh;

edxr_status edxr_load_obj(const char* path, const float pos[3], const float scale[3], const float rot_deg[3],
                          edxr_obj_mesh** mesh);
void edxr_free_obj(edxr_obj_mesh* mesh);

/* Renderer::RenderMesh, Renderer.cpp:100-118: clear, then render one mesh. */
edxr_status edxr_render(edxr_renderer* r, const edxr_mesh* mesh);

/* Wait for enqueued work; re-render after an overflow; report device errors. */
edxr_status edxr_synchronize(edxr_renderer* r);

/* Device pointers of the last frame (synchronizes). */
edxr_status edxr_get_outputs(edxr_renderer* r, edxr_outputs* out);

/* Copy the last frame to host memory; any pointer may be NULL (synchronizes). */
edxr_status edxr_read_outputs(edxr_renderer* r, float* color, float* depth, uint32_t* triangle_id);

/* Renderer::GetBackBuffer (Renderer.cpp:360-363): RGBA8, bottom-up rows,
 * renderer-owned host memory valid until the next call (synchronizes). */
edxr_status edxr_get_back_buffer(edxr_renderer* r, const uint8_t** rgba8);

edxr_status edxr_get_stats(edxr_renderer* r, edxr_stats* stats);

/* Stage timing (no counterpart in the reference, whose viewer only shows fps,
 * RealtimeViewer/Main.cpp:77-84).  While enabled, every pass is launched
 * without graph replay and CUDA events are recorded on the renderer's stream
 * around its stages:
 *   0 clear, 1 vertex transform + clipping + setup + bin count, 2 bin scan,
 *   3 bin scatter, 4 raster + shade (coverage, depth test, the winner's
 *   shading and the output writes).
 * edxr_get_stage_times synchronizes and writes the last pass's milliseconds
 * per stage into ms[0..*count-1] (capacity given in *count on entry). */
edxr_status edxr_set_profiling(edxr_renderer* r, int enable);
edxr_status edxr_get_stage_times(edxr_renderer* r, float* ms, uint32_t* count);

/* Launch tunables (no counterpart in the reference); they change speed only,
 * never results.  The project's autotuner (edxraster_gb300/autotune.py)
 * times candidates on a workload and stores the best as JSON. */
typedef struct edxr_tuning
{
    int small_region;             /* bin entries whose pixel region in a 16x16 tile is at most this
                                     many pixels are rasterized one triangle per thread; 0 disables */
    int raster_variant;           /* 0: raster kernel with the triangle-parallel path, 3 blocks per SM
                                        (85 registers a thread, no spills);
                                     1: the same capped for 5 blocks per SM;
                                     2: pixel-parallel only (small_region ignored), capped for 6 */
    int bin_blocks_per_sm;        /* grid of the per-triangle binning kernels */
    int raster_blocks_per_sm;     /* persistent raster blocks per SM; 0 = the occupancy maximum */
    uint32_t bin_entries_per_triangle;  /* initial bin-buffer capacity per triangle (grows on overflow) */
    int item_entries;             /* bin entries per raster work item (32..1024, default 128): a tile with
                                     more is split over several items that merge their keys; items of at
                                     least 3/4 of it are handed out first */
} edxr_tuning;

edxr_status edxr_set_tuning(edxr_renderer* r, const edxr_tuning* tuning);
edxr_status edxr_get_tuning(edxr_renderer* r, edxr_tuning* tuning);

/* Failure test of the binning scan's bounded wait; no counterpart in the
 * reference, whose binning has no wait and no overflow check (Tile.h:34).
 * Block `block` of the tile-count scan (blocks of 1024 tiles in launch
 * order; -1 = none, the default) keeps its sums to itself, so the block
 * after it waits `spin_limit` polls (0 = the default limit, about a second)
 * and gives up: the frame fails with EDXR_ERR_TIMEOUT instead of hanging,
 * and the renderer stays usable. */
edxr_status edxr_debug_scan_stall(edxr_renderer* r, int block, int spin_limit);

/* Message of the last failing call on this thread. */
const char* edxr_last_error_string(void);

/* ---- batched form: many meshes and views in one launch sequence --------- */

typedef struct edxr_view
{
    uint32_t mesh;            /* index into the mesh array          */
    float mv[16], proj[16], raster[16];
    edxr_shader_params shading;
    int ps_kind;              /* edxr_ps_kind                       */
    int depth_func;           /* edxr_depth_func                    */
} edxr_view;

typedef struct edxr_batch_outputs
{
    float* color;             /* num_views*height*width*4 */
    float* depth;             /* num_views*height*width   */
    uint32_t* triangle_id;    /* num_views*height*width   */
    uint32_t num_views, width, height;
} edxr_batch_outputs;

/* Render every view (same width and height) in one persistent pass: the
 * meshes are read from device memory, views are (mesh, camera) pairs, and the
 * per-view images are bit-identical to edxr_render of the same mesh and
 * camera.  The renderer's state (hierarchical flag) applies to all views. */
edxr_status edxr_render_batched(edxr_renderer* r, const edxr_mesh* meshes, uint32_t num_meshes,
                                const edxr_view* views, uint32_t num_views,
                                uint32_t width, uint32_t height);

edxr_status edxr_get_batch_outputs(edxr_renderer* r, edxr_batch_outputs* out);

/* Copy views [first_view, first_view + num_views) of the last batched pass
 * to host memory; any pointer may be NULL (synchronizes). */
edxr_status edxr_read_batch_outputs(edxr_renderer* r, uint32_t first_view, uint32_t num_views, float* color,
                                    float* depth, uint32_t* triangle_id);

/* ---- differentiable form -------------------------------------------------- */

/* Gradient outputs, device memory; NULL members are skipped.  The adjoint
 * ACCUMULATES into them (the caller zeroes them). */
typedef struct edxr_grads
{
    float* albedo;     /* num_vertices*3 */
    float* normals;    /* num_vertices*3 */
    float* positions;  /* num_vertices*3 */
    float* light;      /* 3 (gradient w.r.t. the unnormalised light vector) */
    float* ks;         /* 1 */
    float* shininess;  /* 1 */
} edxr_grads;

/* Shade the visible surface of the last pass (edxr_render or
 * edxr_render_batched) again, with visibility (the triangle-id buffer) held
 * fixed and perspective-correct barycentrics taken from the un-snapped
 * clip-space vertices of `mesh` (device memory, same sizes as the rendered
 * mesh), writing RGBA32F into color_out (device, frames*height*width*4).
 * Cameras come from the pass; light, ks and shininess from `params`, or from
 * each frame when params is NULL.  This is the forward function whose
 * gradient edxr_backward computes (synchronizes). */
edxr_status edxr_shade_visible(edxr_renderer* r, const edxr_mesh* mesh, const edxr_shader_params* params,
                               float* color_out);

/* Adjoint of edxr_shade_visible: given dL/dcolor (device, same layout,
 * alpha ignored) accumulate dL/d{albedo, normals, positions, light, ks,
 * shininess}.  Recomputes everything per pixel from the triangle-id buffer;
 * no per-pixel intermediates are stored by the forward pass.  Asynchronous
 * on the renderer's stream. */
edxr_status edxr_backward(edxr_renderer* r, const edxr_mesh* mesh, const edxr_shader_params* params,
                          const float* grad_color, const edxr_grads* grads);

/* ---- rendering without device allocation ---------------------------------- */

/* No counterpart in the reference.  One frame for callers that cannot
 * allocate device memory: hosts that own all device memory and give the
 * renderer a fixed budget (engines, plugin hosts), and latency-bound loops
 * that must not call cudaMalloc / cudaFree, which synchronise the device.
 * The caller passes the mesh (device memory), the camera, the state and the
 * shader, and the three output images (device memory, width*height*4 floats,
 * width*height floats, width*height u32).  Every intermediate buffer lives in
 * one fixed file-scope device array (about 24 MiB, held by every GPU that
 * loads the library until exit); nothing is allocated.  Limits: 65536
 * vertices, 65536 triangles, 4096 pixels per side and 2^20 pixels; larger
 * requests fail with EDXR_ERR_INVALID_ARG, and a frame whose bins or clipped
 * polygons do not fit fails with EDXR_ERR_OVERFLOW (the array cannot grow,
 * so the frame is not rendered again; the next call renders normally).  The
 * first call on a device looks the array up with cudaGetSymbolAddress.
 * Calls share the array and keep its contents; calls whose GPU work
 * overlaps race, so serialise them.  Every
 * call blocks the calling thread until its frame on `stream` (a cudaStream_t,
 * NULL = legacy default stream) has finished and its status is read back. */
edxr_status edxr_render_noalloc(const edxr_mesh* mesh, const float mv[16], const float proj[16],
                                const float raster[16], const edxr_state* state, int ps_kind,
                                const edxr_shader_params* params, uint32_t width, uint32_t height,
                                float* color, float* depth, uint32_t* triangle_id, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* EDXR_H */
