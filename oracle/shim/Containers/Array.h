// Growable array with the members the EDXRaster core calls: Add, Size,
// Clear (keeps storage), Resize, Insert(ptr, count, pos), Data, operator[],
// range-for (Renderer.cpp:122-123,183-245; Clipper.h:26-33,96-151;
// FrameBuffer.cpp:25-27; InputBuffer.h:151-189).
// Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

#include <vector>

namespace EDX
{
	template<typename T>
	class Array
	{
		std::vector<T> mData;

	public:
		Array() {}
		int Size() const { return (int)mData.size(); }
		void Add(const T& v) { mData.push_back(v); }
		void Add(T&& v) { mData.push_back(std::move(v)); }
		void Clear() { mData.clear(); }
		void Resize(int n) { mData.resize((size_t)n); }
		void Insert(const T* p, int count, int pos) { mData.insert(mData.begin() + pos, p, p + count); }
		T* Data() { return mData.data(); }
		const T* Data() const { return mData.data(); }
		T& operator[](int i) { return mData[(size_t)i]; }
		const T& operator[](int i) const { return mData[(size_t)i]; }
		typename std::vector<T>::iterator begin() { return mData.begin(); }
		typename std::vector<T>::iterator end() { return mData.end(); }
		typename std::vector<T>::const_iterator begin() const { return mData.begin(); }
		typename std::vector<T>::const_iterator end() const { return mData.end(); }
	};
}
