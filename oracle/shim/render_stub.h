// Test infrastructure: headless stand-in for the reference's render.h.
//
// The reference's demo4.cpp:453-560 fills a draw command buffer for OpenGL;
// that path is out of scope for the oracle.  This header pre-empts
// NBodySimulation/render.h (by defining its include guard) with no-op
// functions of the same names and parameter lists, so demo4.cpp compiles
// without the font, chart and OpenGL headers.  Nothing here is ever called
// by the oracle.
#ifndef SPH_ORACLE_RENDER_STUB_H
#define SPH_ORACLE_RENDER_STUB_H
#define RENDER_H 1

#include <stddef.h>
#include <stdint.h>

namespace Render {
	struct CommandBuffer {};
	typedef void *TextureHandle;
	struct ClipRect {};
	enum class PrimitiveType { Points, Triangles };

	inline void PushRectangle(CommandBuffer *, const Vec2f &, const Vec2f &, const Vec4f &, const bool, const float = 1.0f) {}
	inline void PushLine(CommandBuffer *, const Vec2f &, const Vec2f &, const Vec4f &, const float) {}
	inline void PushCircle(CommandBuffer *, Vec2f, const float, const Vec4f &, const bool, const float = 1.0f) {}
	inline void PushPolygonFrom(CommandBuffer *, Vec2f *, const size_t, const Vec4f &, bool, const float = 1.0f) {}
	inline void PushVertexIndexArrayHeader(CommandBuffer *, uint32_t, void *, uint32_t, void *, uint32_t, void *, uint32_t, void *) {}
	inline void PushVertexIndexArrayDraw(CommandBuffer *, PrimitiveType, uint32_t, float, TextureHandle, const ClipRect &, bool) {}
}

#endif
