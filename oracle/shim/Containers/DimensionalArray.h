// N-dimensional array used by the framebuffer (FrameBuffer.h:8-9,16-18;
// FrameBuffer.cpp:19-27,41,62,76-86,97-103).  Index (i0, i1, i2) is stored
// at i0 + d0 * (i1 + d1 * i2): the first index varies fastest, so a
// (samples, width, height) colour buffer with one sample is a plain
// row-major image.  Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

#include <vector>

namespace EDX
{
	template<int N, typename T>
	class DimensionalArray;

	template<typename T>
	class DimensionalArray<2, T>
	{
		std::vector<T> mData;
		int mDim[2] = { 0, 0 };

	public:
		void Init(const Vector2i& d) { mDim[0] = d.x; mDim[1] = d.y; mData.assign((size_t)d.x * d.y, T()); }
		void Free() { mData.clear(); mData.shrink_to_fit(); mDim[0] = mDim[1] = 0; }
		void Clear() { std::fill(mData.begin(), mData.end(), T()); }
		int LinearSize() const { return (int)mData.size(); }
		Vector2i Index(int i) const { return Vector2i(i % mDim[0], i / mDim[0]); }
		T& operator[](const Vector2i& i) { return mData[(size_t)i.x + (size_t)mDim[0] * i.y]; }
		T& operator[](int i) { return mData[(size_t)i]; }
		const T& operator[](int i) const { return mData[(size_t)i]; }
		T* Data() { return mData.data(); }
		const T* Data() const { return mData.data(); }
	};

	template<typename T>
	class DimensionalArray<3, T>
	{
		std::vector<T> mData;
		int mDim[3] = { 0, 0, 0 };

	public:
		void Init(const Vector3i& d)
		{
			mDim[0] = d.x; mDim[1] = d.y; mDim[2] = d.z;
			mData.assign((size_t)d.x * d.y * d.z, T());
		}
		void Free() { mData.clear(); mData.shrink_to_fit(); mDim[0] = mDim[1] = mDim[2] = 0; }
		void Clear() { std::fill(mData.begin(), mData.end(), T()); }
		int LinearSize() const { return (int)mData.size(); }
		T& operator[](const Vector3i& i) { return mData[(size_t)i.x + (size_t)mDim[0] * ((size_t)i.y + (size_t)mDim[1] * i.z)]; }
		const T& operator[](const Vector3i& i) const { return mData[(size_t)i.x + (size_t)mDim[0] * ((size_t)i.y + (size_t)mDim[1] * i.z)]; }
		T& operator[](int i) { return mData[(size_t)i]; }
		const T& operator[](int i) const { return mData[(size_t)i]; }
		T* Data() { return mData.data(); }
		const T* Data() const { return mData.data(); }
	};
}
