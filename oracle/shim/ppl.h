// Fork-join parallel_for standing in for MSVC PPL (Renderer.cpp:13-14,
// Clipper.h:4,78, FrameBuffer.cpp:5).  A fixed pool of worker threads pulls
// indices from a shared counter; the call returns when every index ran.
// Iterations of every reference call site are independent, so scheduling
// order does not change results.  Test-infrastructure shim.
#pragma once

#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace concurrency
{
	class shim_pool
	{
		std::vector<std::thread> mWorkers;
		std::mutex mMutex;
		std::condition_variable mWake, mDone;
		const std::function<void(int)>* mJob = nullptr;
		std::atomic<int> mNext{ 0 };
		int mFirst = 0, mLast = 0, mActive = 0;
		unsigned mGeneration = 0;
		bool mStop = false;

		void RunChunk()
		{
			for (;;)
			{
				int i = mNext.fetch_add(1);
				if (i >= mLast) break;
				(*mJob)(i);
			}
		}
		void Worker()
		{
			unsigned seen = 0;
			for (;;)
			{
				{
					std::unique_lock<std::mutex> lk(mMutex);
					mWake.wait(lk, [&] { return mStop || mGeneration != seen; });
					if (mStop) return;
					seen = mGeneration;
				}
				RunChunk();
				std::lock_guard<std::mutex> lk(mMutex);
				if (--mActive == 0) mDone.notify_all();
			}
		}

	public:
		explicit shim_pool(int n)
		{
			for (int i = 0; i < n; i++) mWorkers.emplace_back([this] { Worker(); });
		}
		~shim_pool()
		{
			{ std::lock_guard<std::mutex> lk(mMutex); mStop = true; }
			mWake.notify_all();
			for (auto& t : mWorkers) t.join();
		}
		void Run(int first, int last, const std::function<void(int)>& f)
		{
			std::unique_lock<std::mutex> lk(mMutex);
			mJob = &f; mFirst = first; mLast = last; mNext = first;
			mActive = (int)mWorkers.size();
			mGeneration++;
			lk.unlock();
			mWake.notify_all();
			RunChunk();
			lk.lock();
			mDone.wait(lk, [&] { return mActive == 0; });
		}
		static shim_pool& Instance()
		{
			static shim_pool pool(PoolSize());
			return pool;
		}
		static int PoolSize()
		{
			int n = (int)std::thread::hardware_concurrency();
			if (const char* e = std::getenv("EDXR_REF_THREADS")) n = std::atoi(e);
			return n > 1 ? n - 1 : 0;
		}
	};

	template<typename F>
	inline void parallel_for(int first, int last, F&& f)
	{
		if (last <= first) return;
		if (last - first == 1) { f(first); return; }
		std::function<void(int)> job = [&](int i) { f(i); };
		shim_pool::Instance().Run(first, last, job);
	}
}
