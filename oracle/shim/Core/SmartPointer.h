// Owning pointer used by Renderer.h:18-22, Mesh.h:20-23 and Scene.h:13.
// Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

#include <memory>

namespace EDX
{
	template<typename T>
	class UniquePtr
	{
		std::unique_ptr<T> mPtr;
		template<typename U> friend class UniquePtr;

	public:
		UniquePtr() {}
		explicit UniquePtr(T* p) : mPtr(p) {}
		UniquePtr(UniquePtr&& o) : mPtr(std::move(o.mPtr)) {}
		template<typename U>
		UniquePtr(UniquePtr<U>&& o) : mPtr(std::move(o.mPtr)) {}
		UniquePtr& operator=(UniquePtr&& o) { mPtr = std::move(o.mPtr); return *this; }
		template<typename U>
		UniquePtr& operator=(UniquePtr<U>&& o) { mPtr = std::move(o.mPtr); return *this; }
		UniquePtr(const UniquePtr&) = delete;
		UniquePtr& operator=(const UniquePtr&) = delete;

		T* Get() const { return mPtr.get(); }
		void Reset(T* p) { mPtr.reset(p); }
		T* operator->() const { return mPtr.get(); }
		T& operator*() const { return *mPtr; }
		explicit operator bool() const { return (bool)mPtr; }
		bool operator!() const { return !mPtr; }
	};

	template<typename T, typename... Args>
	inline UniquePtr<T> MakeUnique(Args&&... args)
	{
		return UniquePtr<T>(new T(std::forward<Args>(args)...));
	}
}
