// C++ facade of the GB300 pipeline with the interface of EDXRaster's
// Renderer (EDXRaster/Core/Renderer.h:15-59), header-only, over the C ABI of
// edxr.h.  Method names and argument meaning follow the reference; where the
// reference returns nothing and ignores failures, these throw edxr::Error.
#pragma once

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "../edxr.h"

namespace edxr {

class Error : public std::runtime_error
{
public:
    Error(edxr_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    edxr_status status;
};

inline void Check(edxr_status s)
{
    if (s != EDXR_OK)
        throw Error(s, edxr_last_error_string());
}

}  // namespace edxr

namespace EDX {
namespace RasterRenderer {

// Shader choices (Shader.h:37-50, 185-282).  Virtual shader objects cannot run
// inside the kernels, so each class names a device shader and its parameters.
struct DefaultVertexShader
{
    static constexpr int Kind = EDXR_VS_DEFAULT;
};
struct PixelShader
{
    int kind;
    edxr_shader_params params;
};
// BlinnPhongPixelShader as written in the reference: ks 3, exponent 200, no clamp.
inline PixelShader BlinnPhongPixelShader(float lx = 1.0f, float ly = 1.0f, float lz = -1.0f)
{
    return PixelShader{ EDXR_PS_BLINN_PHONG_REFERENCE, { { lx, ly, lz }, 3.0f, 200.0f } };
}
// The Blinn-Phong model of this build: per-vertex albedo, clamped N.H.
inline PixelShader AlbedoBlinnPhongPixelShader(float lx, float ly, float lz, float ks, float shininess)
{
    return PixelShader{ EDXR_PS_BLINN_PHONG, { { lx, ly, lz }, ks, shininess } };
}
inline PixelShader LambertianAlbedoPixelShader(float lx = 1.0f, float ly = 1.0f, float lz = -1.0f)
{
    return PixelShader{ EDXR_PS_LAMBERTIAN_ALBEDO, { { lx, ly, lz }, 0.0f, 1.0f } };
}
inline PixelShader LambertianPixelShader(float lx = 1.0f, float ly = 1.0f, float lz = -1.0f)
{
    return PixelShader{ EDXR_PS_LAMBERTIAN, { { lx, ly, lz }, 0.0f, 1.0f } };
}
// LambertianAlbedoPixelShader as written: the albedo is sampled from the
// triangle's texture slot (Renderer::SetTextures, Mesh::SetTextureIds).
inline PixelShader TexturedLambertianPixelShader(float lx = 1.0f, float ly = 1.0f, float lz = -1.0f)
{
    return PixelShader{ EDXR_PS_LAMBERTIAN_TEXTURED, { { lx, ly, lz }, 0.0f, 1.0f } };
}

enum class TextureFilter { Nearest, Linear, TriLinear, Anisotropic4x, Anisotropic8x, Anisotropic16x };

// Non-owning view of one mesh (Mesh.h:17-69): the buffers stay the caller's.
class Mesh
{
public:
    edxr_mesh desc{};

    // Vertex_PositionNormalTex layout (InputBuffer.h:16-28), 8 floats per vertex.
    static Mesh FromPositionNormalTex(const float* vertices, uint32_t numVertices, const uint32_t* indices,
                                      uint32_t numTriangles, const float* albedo = nullptr,
                                      edxr_memory memory = EDXR_MEMORY_HOST)
    {
        Mesh m;
        m.desc.positions = vertices;
        m.desc.position_stride = 32;
        m.desc.normals = vertices + 3;
        m.desc.normal_stride = 32;
        m.desc.uvs = vertices + 6;
        m.desc.uv_stride = 32;
        m.desc.albedo = albedo;
        m.desc.albedo_stride = 12;
        m.desc.indices = indices;
        m.desc.num_vertices = numVertices;
        m.desc.num_triangles = numTriangles;
        m.desc.memory = memory;
        return m;
    }
    // Separate float3 arrays.
    static Mesh FromArrays(const float* positions, const float* normals, const float* albedo,
                           uint32_t numVertices, const uint32_t* indices, uint32_t numTriangles,
                           edxr_memory memory = EDXR_MEMORY_HOST)
    {
        Mesh m;
        m.desc.positions = positions;
        m.desc.position_stride = 12;
        m.desc.normals = normals;
        m.desc.normal_stride = 12;
        m.desc.albedo = albedo;
        m.desc.albedo_stride = 12;
        m.desc.indices = indices;
        m.desc.num_vertices = numVertices;
        m.desc.num_triangles = numTriangles;
        m.desc.memory = memory;
        return m;
    }
    // Texture coordinates (two floats per vertex) and per-triangle texture
    // slots (Mesh::GetTextureIds, Mesh.h:56-59).
    Mesh& SetTexCoords(const float* uvs, uint32_t strideBytes = 8)
    {
        desc.uvs = uvs;
        desc.uv_stride = strideBytes;
        return *this;
    }
    Mesh& SetTextureIds(const uint32_t* ids)
    {
        desc.texture_ids = ids;
        return *this;
    }
};

class Renderer
{
    edxr_renderer* mpRenderer = nullptr;
    // RenderStates::DefaultSettings (RenderStates.h:55-61)
    edxr_state mState{ EDXR_DEPTH_LEQUAL, 1, 0, EDXR_FILTER_TRILINEAR };
    uint32_t mWidth = 0, mHeight = 0;
    bool mWriteFrames = false;
    int mFrameCount = 0;
    void* mStream = nullptr;
    int mDevice = 0;

public:
    explicit Renderer(int device = 0, void* stream = nullptr) : mStream(stream), mDevice(device) {}
    ~Renderer() { edxr_destroy(mpRenderer); }
    Renderer(const Renderer&) = delete;
    Renderer& operator=(const Renderer&) = delete;

    // Renderer::Initialize (Renderer.cpp:22-62)
    void Initialize(uint32_t width, uint32_t height)
    {
        if (mpRenderer)
        {
            Resize(width, height);
            return;
        }
        edxr_init init{ width, height, mStream, mDevice };
        edxr::Check(edxr_create(&mpRenderer, &init));
        mWidth = width;
        mHeight = height;
        edxr::Check(edxr_set_state(mpRenderer, &mState));
    }
    // Renderer::Resize (Renderer.cpp:64-83)
    void Resize(uint32_t width, uint32_t height)
    {
        edxr::Check(edxr_resize(mpRenderer, width, height));
        mWidth = width;
        mHeight = height;
    }
    // Renderer::SetTransform (Renderer.cpp:85-92): row-major float[16] each.
    void SetTransform(const float* modelView, const float* proj, const float* toRaster)
    {
        edxr::Check(edxr_set_transform(mpRenderer, modelView, proj, toRaster));
    }
    // Renderer::RenderMesh (Renderer.cpp:100-118)
    void RenderMesh(const Mesh& mesh)
    {
        edxr::Check(edxr_render(mpRenderer, &mesh.desc));
        edxr::Check(edxr_synchronize(mpRenderer));
        mFrameCount++;
        if (mWriteFrames)
            WriteFrameToFile();
    }
    // Renderer::WriteFrameToFile (Renderer.cpp:352-358): Frames/FrameNNNNN.bmp
    void WriteFrameToFile() const
    {
        const uint8_t* rgba = GetBackBuffer();
        char name[64];
        std::snprintf(name, sizeof(name), "Frames/Frame%05i.bmp", mFrameCount);
        FILE* f = std::fopen(name, "wb");
        if (!f)
            throw edxr::Error(EDXR_ERR_INVALID_ARG, std::string("cannot open ") + name);
        const uint32_t bytes = 4 * mWidth * mHeight;
        auto put32 = [&](uint32_t v) { for (int i = 0; i < 4; i++) std::fputc((v >> (8 * i)) & 255, f); };
        auto put16 = [&](uint16_t v) { std::fputc(v & 255, f); std::fputc(v >> 8, f); };
        std::fputc('B', f); std::fputc('M', f);
        put32(54 + bytes); put32(0); put32(54);
        put32(40); put32(mWidth); put32(mHeight); put16(1); put16(32);
        for (int i = 0; i < 6; i++) put32(0);
        for (uint32_t i = 0; i < mWidth * mHeight; i++)  // bottom-up rows, BGRA
        {
            std::fputc(rgba[4 * i + 2], f); std::fputc(rgba[4 * i + 1], f);
            std::fputc(rgba[4 * i + 0], f); std::fputc(rgba[4 * i + 3], f);
        }
        std::fclose(f);
    }
    // Renderer::GetBackBuffer (Renderer.cpp:360-363): RGBA8, bottom-up rows.
    const uint8_t* GetBackBuffer() const
    {
        const uint8_t* p = nullptr;
        edxr::Check(edxr_get_back_buffer(mpRenderer, &p));
        return p;
    }
    // Renderer::SetMSAAMode (Renderer.cpp:94-98): 2^msaaCountLog2 samples per pixel (0..5).
    void SetMSAAMode(int msaaCountLog2)
    {
        edxr_state s = mState;
        s.msaa_log2 = msaaCountLog2;
        edxr::Check(edxr_set_state(mpRenderer, &s));
        mState = s;
    }
    // Texture slots (Mesh::GetTextures / RenderStates::TextureSlots): texels
    // copied, mip chains built on the device.
    void SetTextures(const edxr_texture* textures, uint32_t count)
    {
        edxr::Check(edxr_set_textures(mpRenderer, textures, count));
    }
    void SetTextureFilter(TextureFilter filter)
    {
        mState.texture_filter = (int)filter;
        edxr::Check(edxr_set_state(mpRenderer, &mState));
    }
    void SetHierarchicalRasterize(bool hRas)
    {
        mState.hierarchical = hRas ? 1 : 0;
        edxr::Check(edxr_set_state(mpRenderer, &mState));
    }
    void SetWriteFrames(bool wf) { mWriteFrames = wf; }

    // Additions of the GPU build.
    void SetDepthFunc(edxr_depth_func f)
    {
        mState.depth_func = f;
        edxr::Check(edxr_set_state(mpRenderer, &mState));
    }
    void SetPixelShader(const PixelShader& ps)
    {
        edxr::Check(edxr_set_shader(mpRenderer, DefaultVertexShader::Kind, ps.kind, &ps.params));
    }
    edxr_outputs Outputs() const
    {
        edxr_outputs o{};
        edxr::Check(edxr_get_outputs(mpRenderer, &o));
        return o;
    }
    void ReadOutputs(float* color, float* depth, uint32_t* triangleId) const
    {
        edxr::Check(edxr_read_outputs(mpRenderer, color, depth, triangleId));
    }
    edxr_renderer* Handle() const { return mpRenderer; }
};

}  // namespace RasterRenderer
}  // namespace EDX
