/*
 * ORACLE BUILD SHIM -- test infrastructure only.
 *
 * A small functional stand-in for the part of Boost.Thread that openEMS's multithreaded engine
 * and operator use (FDTD/engine_multithread.cpp, FDTD/operator_multithread.cpp): thread,
 * thread_group, barrier, thread_interrupted and this_thread::get_id.  Boost is not installed in
 * this image.  The semantics follow Boost.Thread's documented behaviour, built on the C++ standard
 * library:
 *   - a thread runs a copy of its functor; a boost::thread_interrupted escaping the functor ends
 *     the thread quietly, as Boost's thread entry does;
 *   - thread_group owns its threads; interrupt_all() requests interruption of each, join_all()
 *     joins them;
 *   - barrier::wait() blocks until `count` threads arrived, then releases all of them and resets
 *     (one thread gets `true`); it is an interruption point: a thread whose interruption was
 *     requested throws boost::thread_interrupted from wait(), on entry or while waiting.
 */
#ifndef OEMS_SHIM_BOOST_THREAD_HPP
#define OEMS_SHIM_BOOST_THREAD_HPP

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace boost {

class thread_interrupted {};

namespace oems_shim_detail {
inline std::atomic<bool>*& current_interrupt_flag()
{
	static thread_local std::atomic<bool>* flag = nullptr;
	return flag;
}
inline bool interruption_requested()
{
	std::atomic<bool>* f = current_interrupt_flag();
	return f && f->load();
}
}

class thread
{
public:
	typedef std::thread::id id;

	template <class F>
	explicit thread(F f) : m_flag(std::make_shared<std::atomic<bool>>(false))
	{
		std::shared_ptr<std::atomic<bool>> flag = m_flag;
		m_thread = std::thread([flag, f]() mutable {
			oems_shim_detail::current_interrupt_flag() = flag.get();
			try {
				f();
			} catch (const thread_interrupted&) {
			}
		});
	}
	~thread()
	{
		if (m_thread.joinable())
			m_thread.join();
	}
	thread(const thread&) = delete;
	thread& operator=(const thread&) = delete;

	void interrupt() { m_flag->store(true); }
	void join()
	{
		if (m_thread.joinable())
			m_thread.join();
	}
	bool joinable() const { return m_thread.joinable(); }
	id get_id() const { return m_thread.get_id(); }
	static unsigned int hardware_concurrency() { return std::thread::hardware_concurrency(); }

private:
	std::shared_ptr<std::atomic<bool>> m_flag;
	std::thread m_thread;
};

namespace this_thread {
inline thread::id get_id() { return std::this_thread::get_id(); }
}

class thread_group
{
public:
	thread_group() {}
	~thread_group()
	{
		for (thread* t : m_threads)
			delete t;
	}
	thread_group(const thread_group&) = delete;
	thread_group& operator=(const thread_group&) = delete;

	void add_thread(thread* t)
	{
		std::lock_guard<std::mutex> lk(m_mutex);
		m_threads.push_back(t);
	}
	void interrupt_all()
	{
		std::lock_guard<std::mutex> lk(m_mutex);
		for (thread* t : m_threads)
			t->interrupt();
	}
	void join_all()
	{
		std::lock_guard<std::mutex> lk(m_mutex);
		for (thread* t : m_threads)
			t->join();
	}
	size_t size() const { return m_threads.size(); }

private:
	std::mutex m_mutex;
	std::vector<thread*> m_threads;
};

class barrier
{
public:
	explicit barrier(unsigned int count) : m_count(count), m_waiting(0), m_generation(0) {}
	barrier(const barrier&) = delete;
	barrier& operator=(const barrier&) = delete;

	bool wait()
	{
		std::unique_lock<std::mutex> lk(m_mutex);
		if (oems_shim_detail::interruption_requested())
			throw thread_interrupted();
		unsigned long gen = m_generation;
		if (++m_waiting == m_count) {
			m_waiting = 0;
			++m_generation;
			m_cv.notify_all();
			return true;
		}
		while (gen == m_generation) {
			/* a bounded wait, so that an interruption request is seen while blocked */
			m_cv.wait_for(lk, std::chrono::milliseconds(2));
			if (gen == m_generation && oems_shim_detail::interruption_requested()) {
				--m_waiting;
				throw thread_interrupted();
			}
		}
		return false;
	}

private:
	std::mutex m_mutex;
	std::condition_variable m_cv;
	unsigned int m_count, m_waiting;
	unsigned long m_generation;
};

} // namespace boost

#endif
