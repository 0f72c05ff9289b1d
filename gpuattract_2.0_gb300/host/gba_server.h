/*
 * gba_server.h -- the request interface of the docking energy service, in C++.
 *
 * Same names, argument meaning and error behaviour as the reference's
 * client/service contract, so a caller written against it keeps working:
 *   GenericTypes / Request / WorkItem      src/model/GenericTypes.h, src/server/Request.h,
 *                                          src/server/WorkItem.h
 *   Allocator                              src/allocator/Allocator.h:16-45
 *   Service::createItemProcessor / createDistributor   src/service/Service.h:24-70
 *   Server::submit / wait / createWorkers / setItemSize / setWaitTime
 *                                          src/server/Server.h:49-80, Server.tpp:95-180
 * The implementation is this library's own: a request is copied into
 * server-owned buffers from the service's allocators, split into work items
 * of itemSize poses, and worker threads (one item processor each, created by
 * createWorkers) drain a shared queue.  An item processor returning true is
 * called again with nullptr until it returns false (the reference's drain
 * protocol, src/server/Worker.tpp:14-35).  wait() polls the items every
 * millisecond and gives up after waitTime ms.  Exceptions thrown by a
 * processor are carried to wait() instead of ending the worker.
 */
#ifndef GBA_SERVER_H_
#define GBA_SERVER_H_

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace gba {
namespace host {

constexpr unsigned DEFAULT_ITEM_SIZE = 100;         /* src/server/Server.h:39 */
constexpr unsigned MAX_WAIT_MILLISECONDS = 20000;   /* src/server/Server.h:40 */

using workerId_t = int;

template <typename Input, typename Common, typename Result>
struct GenericTypes {
	using input_t = Input;
	using common_t = Common;
	using result_t = Result;
};

template <typename T>
class Allocator {
public:
	virtual ~Allocator() {}
	virtual T* allocate(size_t size) = 0;
	virtual void deallocate(T* buffer, size_t size = 0) = 0;
};

template <typename T>
class HostAllocator : public Allocator<T> {
public:
	T* allocate(size_t size) override { return new T[size]; }
	void deallocate(T* buffer, size_t) override { delete[] buffer; }
};

template <typename Input, typename Common>
class Request {
public:
	Request() = default;
	Request(Input* data, size_t size, Common common) : _data(data), _size(size), _common(common) {}
	size_t size() const noexcept { return _size; }
	Input* data() const noexcept { return _data; }
	Common common() const noexcept { return _common; }
	void setDataAndSize(Input* data, size_t size) noexcept { _data = data; _size = size; }
	void setCommon(Common const& common) noexcept { _common = common; }
	void reset() { _data = nullptr; _size = 0; _common = Common(); }

private:
	Input* _data = nullptr;
	size_t _size = 0;
	Common _common{};
};

template <typename Input, typename Common, typename Result>
class WorkItem {
public:
	WorkItem() : _processed(false) {}
	WorkItem(Input* in, unsigned size, Common* common, Result* out)
		: _in(in), _size(size), _common(common), _out(out), _processed(false) {}
	WorkItem(WorkItem const&) = delete;
	WorkItem& operator=(WorkItem const&) = delete;

	unsigned size() const noexcept { return _size; }
	Input* inputBuffer() const noexcept { return _in; }
	Common* common() const noexcept { return _common; }
	Result* resultBuffer() const noexcept { return _out; }
	void setProcessed() noexcept { _processed.store(true, std::memory_order_release); }
	bool isProcessed() const noexcept { return _processed.load(std::memory_order_acquire); }
	bool isValid() const noexcept { return _in && _size > 0 && _common && _out; }

	/* an exception from the item processor, reported by Server::wait */
	void setError(std::string const& e) { _error = e; }
	std::string const& error() const noexcept { return _error; }

private:
	Input* _in = nullptr;
	unsigned _size = 0;
	Common* _common = nullptr;
	Result* _out = nullptr;
	std::atomic<bool> _processed;
	std::string _error;
};

template <typename GT>
class Service {
public:
	using genericTypes_t = GT;
	using input_t = typename GT::input_t;
	using common_t = typename GT::common_t;
	using result_t = typename GT::result_t;
	using workItem_t = WorkItem<input_t, common_t, result_t>;
	using itemProcessor_t = std::function<bool(workItem_t*)>;
	using distributor_t = std::function<std::vector<workerId_t>(common_t const*, size_t)>;

	Service(std::shared_ptr<Allocator<input_t>> in, std::shared_ptr<Allocator<result_t>> out)
		: _in(std::move(in)), _out(std::move(out)) {}
	virtual ~Service() {}
	void setInputAllocator(std::shared_ptr<Allocator<input_t>> a) { _in = std::move(a); }
	void setResultAllocator(std::shared_ptr<Allocator<result_t>> a) { _out = std::move(a); }
	Allocator<input_t>* getInputAllocator() { return _in.get(); }
	Allocator<result_t>* getResultAllocator() { return _out.get(); }

	virtual itemProcessor_t createItemProcessor() = 0;
	/* Workers allowed to take items of a given common block (all by default). */
	virtual distributor_t createDistributor() {
		return [](common_t const*, size_t n) {
			std::vector<workerId_t> ids(n);
			for (size_t i = 0; i < n; ++i) ids[i] = (workerId_t)i;
			return ids;
		};
	}

private:
	std::shared_ptr<Allocator<input_t>> _in;
	std::shared_ptr<Allocator<result_t>> _out;
};

template <typename GT>
class Server {
public:
	using service_t = Service<GT>;
	using input_t = typename GT::input_t;
	using result_t = typename GT::result_t;
	using common_t = typename GT::common_t;
	using workItem_t = typename service_t::workItem_t;
	using request_t = Request<input_t, common_t>;

	explicit Server(std::shared_ptr<service_t> service) { setService(service); }
	Server(Server const&) = delete;

	~Server() {
		stopWorkers();
		for (auto& kv : _requests) releaseBuffers(*kv.second);
		for (auto& st : _orphans) releaseBuffers(*st);
	}

	std::shared_ptr<service_t> service() noexcept { return _service; }

	void setService(std::shared_ptr<service_t> const& service) {
		if (service.get() == nullptr) throw std::invalid_argument("Invalid service (nullptr).");
		if (!service->getInputAllocator() || !service->getResultAllocator())
			throw std::invalid_argument("Invalid service allocators (nullptr).");
		_service = service;
	}

	void createWorkers(unsigned number) {
		stopWorkers();
		_stop = false;
		for (unsigned i = 0; i < number; ++i) {
			auto fn = _service->createItemProcessor();
			_workers.emplace_back([this, fn] { workerLoop(fn); });
		}
	}

	void setWaitTime(unsigned milliSeconds) noexcept { _waitTime = milliSeconds; }

	void setItemSize(size_t itemSize) {
		if (itemSize == 0) throw std::invalid_argument("Item size must be greater than zero.");
		_itemSize = itemSize;
	}

	size_t itemSize() const noexcept { return _itemSize; }

	void submit(request_t& req) {
		std::lock_guard<std::mutex> g(_reqMu);
		if (_requests.count(&req)) throw std::invalid_argument("Request has already been submitted.");
		if (req.data() == nullptr) throw std::invalid_argument("Invalid input buffer (nullptr).");
		auto st = std::make_unique<State>();
		st->size = req.size();
		st->common = req.common();
		if (st->size > 0) {
			st->in = _service->getInputAllocator()->allocate(st->size);
			st->out = _service->getResultAllocator()->allocate(st->size);
			std::copy(req.data(), req.data() + st->size, st->in);
			const size_t nitems = (st->size + _itemSize - 1) / _itemSize;
			st->items.reserve(nitems);
			for (size_t k = 0; k < nitems; ++k) {
				const size_t b = k * _itemSize, e = std::min(st->size, b + _itemSize);
				st->items.emplace_back(new workItem_t(st->in + b, (unsigned)(e - b), &st->common, st->out + b));
			}
			{
				std::lock_guard<std::mutex> q(_qMu);
				for (auto& it : st->items) _queue.push_back(it.get());
			}
			_qCv.notify_all();
		}
		_requests.emplace(&req, std::move(st));
		req.reset();
	}

	void wait(request_t const& req, result_t* result) {
		State* st = nullptr;
		{
			std::lock_guard<std::mutex> g(_reqMu);
			auto it = _requests.find(&req);
			if (it == _requests.end() || result == nullptr)
				throw std::invalid_argument(
						"Either request has not been submitted or clientBuffer invalid (nullptr).");
			st = it->second.get();
		}
		unsigned count = 0;
		bool processed;
		while (!(processed = allProcessed(*st)) && count < _waitTime) {
			++count;
			std::this_thread::sleep_for(std::chrono::milliseconds(1));
		}
		std::string err;
		for (auto& it : st->items)
			if (it->isProcessed() && !it->error().empty()) err = it->error();
		if (processed && err.empty() && st->size > 0) std::copy(st->out, st->out + st->size, result);
		bool retire = processed;
		if (!processed) {
			/* a timed-out request keeps its buffers until its items finish; the
			 * server drops queued ones so no worker touches them afterwards */
			std::lock_guard<std::mutex> q(_qMu);
			for (auto& it : st->items)
				for (auto qi = _queue.begin(); qi != _queue.end();)
					qi = (*qi == it.get()) ? _queue.erase(qi) : qi + 1;
		}
		{
			std::lock_guard<std::mutex> g(_reqMu);
			auto node = _requests.extract(&req);
			if (retire) releaseBuffers(*node.mapped());
			else _orphans.push_back(std::move(node.mapped()));
		}
		if (!processed) throw std::runtime_error("Request takes too long to finish for unknown reasons");
		if (!err.empty()) throw std::runtime_error(err);
	}

private:
	struct State {
		size_t size = 0;
		common_t common{};
		input_t* in = nullptr;
		result_t* out = nullptr;
		std::vector<std::unique_ptr<workItem_t>> items;
	};

	static bool allProcessed(State const& st) {
		for (auto& it : st.items)
			if (!it->isProcessed()) return false;
		return true;
	}

	void releaseBuffers(State& st) {
		if (st.in) _service->getInputAllocator()->deallocate(st.in, st.size);
		if (st.out) _service->getResultAllocator()->deallocate(st.out, st.size);
		st.in = nullptr;
		st.out = nullptr;
	}

	void workerLoop(typename service_t::itemProcessor_t fn) {
		bool callAgain = false;
		for (;;) {
			workItem_t* item = nullptr;
			{
				std::unique_lock<std::mutex> q(_qMu);
				if (!callAgain) _qCv.wait(q, [this] { return _stop || !_queue.empty(); });
				if (_queue.empty() && _stop && !callAgain) return;
				if (!_queue.empty()) {
					item = _queue.front();
					_queue.pop_front();
				}
			}
			try {
				callAgain = fn(item);
			} catch (std::exception const& e) {
				callAgain = false;
				if (item) {
					item->setError(e.what());
					item->setProcessed();
				}
			}
			if (_stop && !callAgain) {
				std::lock_guard<std::mutex> q(_qMu);
				if (_queue.empty()) return;
			}
		}
	}

	void stopWorkers() {
		{
			std::lock_guard<std::mutex> q(_qMu);
			_stop = true;
		}
		_qCv.notify_all();
		for (auto& t : _workers) t.join();
		_workers.clear();
	}

	std::shared_ptr<service_t> _service;
	size_t _itemSize = DEFAULT_ITEM_SIZE;
	unsigned _waitTime = MAX_WAIT_MILLISECONDS;
	std::mutex _reqMu;
	std::map<request_t const*, std::unique_ptr<State>> _requests;
	std::vector<std::unique_ptr<State>> _orphans;
	std::mutex _qMu;
	std::condition_variable _qCv;
	std::deque<workItem_t*> _queue;
	std::vector<std::thread> _workers;
	bool _stop = false;
};

}  // namespace host
}  // namespace gba

#endif
