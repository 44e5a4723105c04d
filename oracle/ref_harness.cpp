// Harness around the reference's own rasterization pipeline, compiled
// UNMODIFIED from the EDXRaster sources (Core/Renderer.cpp, FrameBuffer.cpp,
// Scene.cpp and the Core/Utils headers) against the project-written EDXUtil
// shim in oracle/shim.  Test infrastructure only: it is the parity anchor for
// the C restatement in oracle/edxr_oracle.c and the timed CPU baseline.  It is
// never linked into, or called by, the product library.
//
// Entry points:
//  * edxr_ref_parity  runs the reference stages in the order RenderMesh runs
//    them (Renderer.cpp:100-118: Clear, VertexProcessing, Clipping,
//    TiledRasterization) and reads back, per pixel, the fragment that the
//    colour resolve would keep (UpdateFrameBuffer, Renderer.cpp:305-350: the
//    last fragment in tile order whose coverage bit is set), its barycentrics,
//    and the final tiled depth value (FrameBuffer.cpp:54-68).  Each input
//    triangle i is given texture id i (Clipper.h:95, RasterTriangle.h:63,
//    Shader.h:112), so the fragment carries the input-triangle index.
//  * edxr_ref_parity_ms  the same with MSAA, per sample.
//  * edxr_ref_time    times the public Renderer::RenderMesh end to end.
#include "EDXPrerequisites.h"
#include "Renderer.h"
#include "FrameBuffer.h"
#include "Rasterizer.h"
#include "Scene.h"
#include "Clipper.h"
#include "../Utils/Mesh.h"
#include "../Utils/InputBuffer.h"

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <vector>

using namespace EDX;
using namespace EDX::RasterRenderer;

// ---------------------------------------------------------------------------
// Access to the renderer's private stages and buffers without editing the
// reference: an explicit instantiation may name private members, and the
// friend function it defines hands the member pointer out.
template<typename Tag, typename Tag::type M>
struct PrivateAccess
{
	friend typename Tag::type Get(Tag) { return M; }
};
#define EDXR_PRIVATE(name, cls, mtype, member) \
	struct name { typedef mtype cls::*type; friend type Get(name); }; \
	template struct PrivateAccess<name, &cls::member>;

EDXR_PRIVATE(R_Tiles, Renderer, Array<Tile>, mTiles)
EDXR_PRIVATE(R_FrameBuffer, Renderer, UniquePtr<FrameBuffer>, mpFrameBuffer)
EDXR_PRIVATE(R_NumCores, Renderer, int, mNumCores)
typedef Array<DimensionalArray<3, FloatSSE>> TiledDepth;
EDXR_PRIVATE(FB_Depth, FrameBuffer, TiledDepth, mTiledDepthBuffer)
EDXR_PRIVATE(FB_TileDimX, FrameBuffer, uint, mTileDimX)

typedef void (Renderer::*VertexProcessingFn)(const IVertexBuffer*);
typedef void (Renderer::*ClippingFn)(IndexBuffer*, const Array<uint>&);
typedef void (Renderer::*TiledRasterizationFn)();
struct R_VertexProcessing { typedef VertexProcessingFn type; friend type Get(R_VertexProcessing); };
template struct PrivateAccess<R_VertexProcessing, &Renderer::VertexProcessing>;
struct R_Clipping { typedef ClippingFn type; friend type Get(R_Clipping); };
template struct PrivateAccess<R_Clipping, &Renderer::Clipping>;
struct R_TiledRasterization { typedef TiledRasterizationFn type; friend type Get(R_TiledRasterization); };
template struct PrivateAccess<R_TiledRasterization, &Renderer::TiledRasterization>;

// ---------------------------------------------------------------------------
// Mesh.cpp is not compiled (it needs the OBJ loader), so this harness gives
// Mesh::LoadMesh its own definition: it serves the synthetic mesh staged in
// gPending instead of reading a file.
namespace
{
	struct PendingMesh
	{
		const float* vertices = nullptr;  // nv x 8 floats: position, normal, uv
		int nv = 0;
		const uint32_t* indices = nullptr;
		int nt = 0;
		bool triangleIdAsTexture = true;
	};
	thread_local PendingMesh gPending;
}

namespace EDX
{
	namespace RasterRenderer
	{
		void Mesh::LoadMesh(const Vector3&, const Vector3&, const Vector3&, const char*)
		{
			mpVertexBuf.Reset(CreateVertexBuffer<Vertex_PositionNormalTex>(gPending.vertices, gPending.nv));
			mpIndexBuf.Reset(CreateIndexBuffer(gPending.indices, gPending.nt));
			mTextures.Clear();
			mTextures.Add(MakeUnique<ConstantTexture2D<Color>>(Color(0.9f)));
			mTexIdx.Resize(gPending.nt);
			for (int i = 0; i < gPending.nt; i++)
				mTexIdx[i] = gPending.triangleIdAsTexture ? (uint)i : 0u;
		}
	}
}

namespace
{
	void SetupRenderer(Renderer& r, int width, int height, const float* mv, const float* proj,
		const float* raster, int hierarchical)
	{
		r.Initialize((uint)width, (uint)height);
		r.SetTransform(Matrix(mv), Matrix(proj), Matrix(raster));
		r.SetHierarchicalRasterize(hierarchical != 0);
	}
}

extern "C" {

// Returns the number of fragments the reference generated (all tiles), or a
// negative value on bad arguments.  Outputs are W*H arrays in top-down raster
// order (row y = raster y): input-triangle id (0xFFFFFFFF where nothing
// passed), final depth, and the winning fragment's two barycentrics.
long long edxr_ref_parity(int width, int height,
	const float* mv16, const float* proj16, const float* raster16,
	const float* vertices, int nv, const uint32_t* indices, int nt,
	int hierarchical,
	uint32_t* outId, float* outDepth, float* outLambda0, float* outLambda1)
{
	if (width <= 0 || height <= 0 || nv < 0 || nt < 0)
		return -1;

	gPending.vertices = vertices;
	gPending.nv = nv;
	gPending.indices = indices;
	gPending.nt = nt;
	gPending.triangleIdAsTexture = true;

	long long fragments = 0;
	{
		Renderer renderer;
		SetupRenderer(renderer, width, height, mv16, proj16, raster16, hierarchical);
		Mesh mesh;
		mesh.LoadMesh(Vector3(), Vector3(), Vector3(), "");

		FrameBuffer* fb = (renderer.*Get(R_FrameBuffer())).Get();
		fb->Clear();
		(renderer.*Get(R_VertexProcessing()))(mesh.GetVertexBuffer());
		(renderer.*Get(R_Clipping()))(mesh.GetIndexBuffer(), mesh.GetTextureIds());
		(renderer.*Get(R_TiledRasterization()))();

		const size_t npix = (size_t)width * height;
		for (size_t i = 0; i < npix; i++)
		{
			outId[i] = 0xFFFFFFFFu;
			outLambda0[i] = 0.0f;
			outLambda1[i] = 0.0f;
		}

		Array<Tile>& tiles = renderer.*Get(R_Tiles());
		for (int t = 0; t < tiles.Size(); t++)
		{
			const Array<Fragment>& frags = tiles[t].fragmentBuf;
			fragments += frags.Size();
			for (int j = 0; j < frags.Size(); j++)
			{
				const Fragment& f = frags[j];
				for (int lane = 0; lane < 4; lane++)
				{
					if (f.coverageMask.GetBit(lane) == 0)
						continue;
					const int x = f.x + (lane & 1);
					const int y = f.y + (lane >> 1);
					if (x >= width || y >= height)
						continue;
					const size_t p = (size_t)y * width + x;
					outId[p] = f.textureId;
					outLambda0[p] = f.lambda0[lane];
					outLambda1[p] = f.lambda1[lane];
				}
			}
		}

		Array<DimensionalArray<3, FloatSSE>>& depth = (*fb).*Get(FB_Depth());
		const int tileDimX = (int)((*fb).*Get(FB_TileDimX()));
		for (int y = 0; y < height; y++)
			for (int x = 0; x < width; x++)
			{
				const int tx = x >> Tile::SIZE_LOG_2, ty = y >> Tile::SIZE_LOG_2;
				const int ix = x & (Tile::SIZE - 1), iy = y & (Tile::SIZE - 1);
				const FloatSSE& q = depth[ty * tileDimX + tx][Vector3i(0, ix >> 1, (Tile::SIZE - 1 - iy) >> 1)];
				outDepth[(size_t)y * width + x] = q[(x & 1) + 2 * (y & 1)];
			}
	}
	return fragments;
}

// The same with 2^msaaLog2 samples per pixel (Renderer::SetMSAAMode,
// Renderer.cpp:94-98): per sample, the input-triangle id of the last fragment
// in tile order whose coverage bit for that sample is set (UpdateFrameBuffer,
// Renderer.cpp:305-350, bit (sId << 2) + lane) and the final tiled depth of
// the sample.  Outputs are S planes of W*H, sample-major.
long long edxr_ref_parity_ms(int width, int height,
	const float* mv16, const float* proj16, const float* raster16,
	const float* vertices, int nv, const uint32_t* indices, int nt,
	int hierarchical, int msaaLog2,
	uint32_t* outId, float* outDepth)
{
	if (width <= 0 || height <= 0 || nv < 0 || nt < 0 || msaaLog2 < 0 || msaaLog2 > 5)
		return -1;

	gPending.vertices = vertices;
	gPending.nv = nv;
	gPending.indices = indices;
	gPending.nt = nt;
	gPending.triangleIdAsTexture = true;

	long long fragments = 0;
	{
		Renderer renderer;
		SetupRenderer(renderer, width, height, mv16, proj16, raster16, hierarchical);
		renderer.SetMSAAMode(msaaLog2);
		Mesh mesh;
		mesh.LoadMesh(Vector3(), Vector3(), Vector3(), "");

		FrameBuffer* fb = (renderer.*Get(R_FrameBuffer())).Get();
		const int S = (int)fb->GetSampleCount();
		fb->Clear();
		(renderer.*Get(R_VertexProcessing()))(mesh.GetVertexBuffer());
		(renderer.*Get(R_Clipping()))(mesh.GetIndexBuffer(), mesh.GetTextureIds());
		(renderer.*Get(R_TiledRasterization()))();

		const size_t npix = (size_t)width * height;
		for (size_t i = 0; i < npix * S; i++)
			outId[i] = 0xFFFFFFFFu;

		Array<Tile>& tiles = renderer.*Get(R_Tiles());
		for (int t = 0; t < tiles.Size(); t++)
		{
			const Array<Fragment>& frags = tiles[t].fragmentBuf;
			fragments += frags.Size();
			for (int j = 0; j < frags.Size(); j++)
			{
				const Fragment& f = frags[j];
				for (int s = 0; s < S; s++)
					for (int lane = 0; lane < 4; lane++)
					{
						if (f.coverageMask.GetBit((s << 2) + lane) == 0)
							continue;
						const int x = f.x + (lane & 1);
						const int y = f.y + (lane >> 1);
						if (x >= width || y >= height)
							continue;
						outId[(size_t)s * npix + (size_t)y * width + x] = f.textureId;
					}
			}
		}

		Array<DimensionalArray<3, FloatSSE>>& depth = (*fb).*Get(FB_Depth());
		const int tileDimX = (int)((*fb).*Get(FB_TileDimX()));
		for (int s = 0; s < S; s++)
			for (int y = 0; y < height; y++)
				for (int x = 0; x < width; x++)
				{
					const int tx = x >> Tile::SIZE_LOG_2, ty = y >> Tile::SIZE_LOG_2;
					const int ix = x & (Tile::SIZE - 1), iy = y & (Tile::SIZE - 1);
					const FloatSSE& q = depth[ty * tileDimX + tx][Vector3i(s, ix >> 1, (Tile::SIZE - 1 - iy) >> 1)];
					outDepth[(size_t)s * npix + (size_t)y * width + x] = q[(x & 1) + 2 * (y & 1)];
				}
	}
	return fragments;
}

// Median wall time (seconds) of `frames` calls to Renderer::RenderMesh after
// `warmup` untimed calls.  All triangles use one constant texture, the
// reference's default pixel shader (LambertianAlbedoPixelShader,
// Renderer.cpp:41) and its 8-bit output.  Returns the core count used in
// *coresUsed.
double edxr_ref_time(int width, int height,
	const float* mv16, const float* proj16, const float* raster16,
	const float* vertices, int nv, const uint32_t* indices, int nt,
	int frames, int warmup, int* coresUsed)
{
	if (width <= 0 || height <= 0 || frames <= 0)
		return -1.0;
	gPending.vertices = vertices;
	gPending.nv = nv;
	gPending.indices = indices;
	gPending.nt = nt;
	gPending.triangleIdAsTexture = false;

	std::vector<double> times;
	{
		Renderer renderer;
		SetupRenderer(renderer, width, height, mv16, proj16, raster16, 1);
		if (coresUsed)
			*coresUsed = renderer.*Get(R_NumCores());
		Mesh mesh;
		mesh.LoadMesh(Vector3(), Vector3(), Vector3(), "");
		for (int i = 0; i < warmup; i++)
			renderer.RenderMesh(mesh);
		for (int i = 0; i < frames; i++)
		{
			auto t0 = std::chrono::steady_clock::now();
			renderer.RenderMesh(mesh);
			auto t1 = std::chrono::steady_clock::now();
			times.push_back(std::chrono::duration<double>(t1 - t0).count());
		}
	}
	std::sort(times.begin(), times.end());
	return times[times.size() / 2];
}

}  // extern "C"
