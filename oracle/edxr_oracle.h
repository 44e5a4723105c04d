/* CPU oracle for the EDXRaster rasterization pipeline (test infrastructure).
 *
 * A plain-C restatement of Renderer::RenderMesh (EDXRaster/Core/Renderer.cpp:
 * 100-118) for one frame: vertex transform, homogeneous clipping, fixed-point
 * triangle setup, 32x32 binning, coarse/fine/trivial-accept rasterization,
 * the depth test, and "last passing fragment wins" colour resolve.  Integer,
 * ordering and depth results are bit-exact with the reference; colour is an
 * FP64 evaluation of the shading model at the winning fragment.
 *
 * Only tests, the smoke check and the benchmark's CPU-baseline leg use this
 * code, and only as the checker.  The product library never links it.
 */
#ifndef EDXR_ORACLE_H
#define EDXR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum
{
    EDXR_ORACLE_DEPTH_LEQUAL = 0, /* FrameBuffer.cpp:64 (reference) */
    EDXR_ORACLE_DEPTH_LESS = 1
};

enum
{
    EDXR_ORACLE_PS_BLINN_PHONG = 0,           /* albedo*diffuse + ks*max(N.H,0)^s */
    EDXR_ORACLE_PS_BLINN_PHONG_REFERENCE = 1, /* Shader.h:249-281: diffuse + ks*(N.H)^s */
    EDXR_ORACLE_PS_LAMBERTIAN_ALBEDO = 2,     /* Shader.h:212-243 with per-vertex albedo */
    EDXR_ORACLE_PS_LAMBERTIAN = 3,            /* Shader.h:188-206 */
    EDXR_ORACLE_PS_LAMBERTIAN_TEXTURED = 4    /* Shader.h:209-244, albedo sampled from the texture */
};

/* One texture slot: texels in rows of `width`, row 0 at v = 0; format 0 =
 * RGBA8 (channel = byte / 255), 1 = RGBA32F. */
typedef struct
{
    int width, height, format;
    const void* texels;
} edxr_oracle_texture;

typedef struct
{
    int width, height;
    float mv[16];     /* row-major, column vectors */
    float proj[16];
    float raster[16];
    int depth_func;   /* EDXR_ORACLE_DEPTH_* */
    int hierarchical; /* RenderStates::HierarchicalRasterize */
    int shader;       /* EDXR_ORACLE_PS_* */
    float light[3];   /* direction towards the light, normalised inside */
    float ks, shininess;
    int threads;      /* worker threads for the per-tile stages (>=1) */
    int msaa_log2;    /* RenderStates::MultiSampleLevel: 0 (one sample) .. 5 (32 samples) */
    const edxr_oracle_texture* textures; /* texture slots of the textured shader */
    int num_textures;
    int texture_filter; /* 0 nearest, 1 linear, 2 trilinear, 3..5 anisotropic 4x/8x/16x */
} edxr_oracle_params;

typedef struct
{
    const float* positions; int position_stride; /* strides in floats */
    const float* normals;   int normal_stride;   /* may be NULL -> 0 */
    const float* uvs;       int uv_stride;       /* may be NULL -> 0 */
    const float* albedo;    int albedo_stride;   /* may be NULL -> 1 */
    const uint32_t* indices;                     /* 3 per triangle */
    int nv, nt;
    const uint32_t* texture_ids;                 /* per triangle, may be NULL -> 0 */
} edxr_oracle_mesh;

/* With S = 1 << msaa_log2 samples, id and depth hold S planes of W*H
 * (sample s at offset s*W*H); the barycentrics are written for S == 1 only.
 * colour is the winner's FP64 shading (S == 1) or the reference's resolve:
 * each sample's winner shaded at the pixel centre and stored as 8 bits, the
 * samples averaged in float (FrameBuffer::Resolve, FrameBuffer.cpp:70-87). */
typedef struct
{
    uint32_t* id;     /* S*W*H input-triangle index of the winner, 0xFFFFFFFF if none */
    float* depth;     /* S*W*H final depth buffer (clear value 1.0) */
    float* lambda0;   /* W*H winner barycentrics (optional) */
    float* lambda1;
    double* color;    /* W*H*4 RGBA, alpha 1 where covered (optional) */
    /* statistics */
    long long fragments;   /* quad fragments emitted */
    long long raster_tris; /* triangles that survived setup */
    long long clipped_input_tris;
    long long bin_refs;
} edxr_oracle_out;

/* Returns 0 on success, negative on invalid arguments or allocation failure. */
int edxr_oracle_render(const edxr_oracle_params* params, const edxr_oracle_mesh* mesh,
                       edxr_oracle_out* out);

/* FP64 evaluation of the shading model at an arbitrary point, exposed so the
 * adjoint tests can difference it.  Inputs are the per-vertex attributes of
 * one triangle, its perspective-correct barycentrics and the eye position. */
void edxr_oracle_shade(const edxr_oracle_params* params, const double b[3],
                       const double pos[3][3], const double nrm[3][3],
                       const double alb[3][3], const double eye[3], double rgb[3]);

#ifdef __cplusplus
}
#endif

#endif
