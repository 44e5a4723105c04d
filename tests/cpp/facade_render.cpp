// Renders one scene through the C++ facade (include/edxr/Renderer.h) the way
// EDXRaster's viewer drives its Renderer (RealtimeViewer/Main.cpp:38-39,71-75),
// and writes the triangle-id, depth and back buffers for the test to compare.
//
// usage: facade_render <scene.bin> <out.bin> [arrays|interleaved] [write]
// scene.bin: u32 width, height, nv, nt; f32 mv[16], proj[16], raster[16];
//            f32 light[3], ks, shininess; f32 positions[nv*3], normals[nv*3],
//            albedo[nv*3]; u32 indices[nt*3]
// out.bin:   u32 ids[w*h]; f32 depth[w*h]; f32 color[w*h*4]; u8 backbuffer[w*h*4]
// "interleaved" hands the mesh over in the reference's own vertex layout,
// Vertex_PositionNormalTex (InputBuffer.h:16-28: position, normal and
// texture coordinate, 32 bytes per vertex), instead of separate arrays;
// "write" turns SetWriteFrames on, so RenderMesh also writes the frame as
// Frames/FrameNNNNN.bmp under the working directory (Renderer.cpp:352-358).
#include <cstdio>
#include <string>
#include <vector>

#include "edxr/Renderer.h"

using namespace EDX::RasterRenderer;

template <typename T>
static void read_all(FILE* f, std::vector<T>& v, size_t n)
{
    v.resize(n);
    if (std::fread(v.data(), sizeof(T), n, f) != n)
        throw std::runtime_error("short read");
}

int main(int argc, char** argv)
{
    if (argc < 3 || argc > 5)
        return 2;
    const bool interleaved = argc > 3 && std::string(argv[3]) == "interleaved";
    const bool write = argc > 4 && std::string(argv[4]) == "write";
    try
    {
        FILE* f = std::fopen(argv[1], "rb");
        if (!f)
            return 3;
        std::vector<uint32_t> hdr;
        read_all(f, hdr, 4);
        const uint32_t W = hdr[0], H = hdr[1], nv = hdr[2], nt = hdr[3];
        std::vector<float> mats, shade, pos, nrm, alb;
        std::vector<uint32_t> idx;
        read_all(f, mats, 48);
        read_all(f, shade, 5);
        read_all(f, pos, 3 * (size_t)nv);
        read_all(f, nrm, 3 * (size_t)nv);
        read_all(f, alb, 3 * (size_t)nv);
        read_all(f, idx, 3 * (size_t)nt);
        std::fclose(f);

        Renderer renderer;
        renderer.Initialize(W, H);
        renderer.SetTransform(&mats[0], &mats[16], &mats[32]);
        renderer.SetPixelShader(AlbedoBlinnPhongPixelShader(shade[0], shade[1], shade[2], shade[3], shade[4]));
        renderer.SetDepthFunc(EDXR_DEPTH_LESS);
        renderer.SetWriteFrames(write);
        std::vector<float> vertices;
        if (interleaved)
        {
            vertices.assign(8 * (size_t)nv, 0.0f);  // texture coordinates stay 0
            for (size_t v = 0; v < nv; v++)
                for (int c = 0; c < 3; c++)
                {
                    vertices[8 * v + c] = pos[3 * v + c];
                    vertices[8 * v + 3 + c] = nrm[3 * v + c];
                }
            renderer.RenderMesh(Mesh::FromPositionNormalTex(vertices.data(), nv, idx.data(), nt, alb.data()));
        }
        else
            renderer.RenderMesh(Mesh::FromArrays(pos.data(), nrm.data(), alb.data(), nv, idx.data(), nt));
        std::vector<uint32_t> ids((size_t)W * H);
        std::vector<float> depth((size_t)W * H), color(4 * (size_t)W * H);
        renderer.ReadOutputs(color.data(), depth.data(), ids.data());
        const uint8_t* bb = renderer.GetBackBuffer();

        bool threw = false;
        try
        {
            renderer.SetMSAAMode(6);  // at most 32 samples: must throw, renderer stays usable
        }
        catch (const edxr::Error& e)
        {
            threw = e.status == EDXR_ERR_INVALID_ARG;
        }
        if (!threw)
            return 4;

        FILE* o = std::fopen(argv[2], "wb");
        std::fwrite(ids.data(), 4, ids.size(), o);
        std::fwrite(depth.data(), 4, depth.size(), o);
        std::fwrite(color.data(), 4, color.size(), o);
        std::fwrite(bb, 1, (size_t)W * H * 4, o);
        std::fclose(o);
    }
    catch (const std::exception& e)
    {
        std::fprintf(stderr, "facade_render: %s\n", e.what());
        return 1;
    }
    return 0;
}
