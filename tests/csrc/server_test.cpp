/* Request-interface tests of gba_server.h, mirroring the reference's own
 * server tests (test/server/Server_Test.cpp): construction and interface
 * errors with their exact messages, the wait timeout with a service that
 * never completes (test/server/Service_TimeOut.cpp), and the split /
 * dispatch / gather sweep with a mock service computing input * common
 * (test/server/Service_Mock.h).  Prints "OK" and exits 0 on success. */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../gpuattract_2.0_gb300/host/gba_server.h"

using namespace gba::host;

static int failures = 0;
#define CHECK(cond)                                                          \
	do {                                                                     \
		if (!(cond)) {                                                       \
			std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond); \
			++failures;                                                      \
		}                                                                    \
	} while (0)

template <typename F>
static std::string error_of(F&& f) {
	try {
		f();
	} catch (std::exception& e) {
		return e.what();
	}
	return "";
}

using MockTypes = GenericTypes<int, int, int>;

class MockService : public Service<MockTypes> {
public:
	explicit MockService(bool allocators = true)
		: Service<MockTypes>(allocators ? std::make_shared<HostAllocator<int>>() : nullptr,
		                      allocators ? std::make_shared<HostAllocator<int>>() : nullptr) {}
	itemProcessor_t createItemProcessor() override {
		return [](workItem_t* item) -> bool {
			if (!item) return false;
			const int c = *item->common();
			for (unsigned i = 0; i < item->size(); ++i) item->resultBuffer()[i] = item->inputBuffer()[i] * c;
			item->setProcessed();
			return false;
		};
	}
};

/* Asks to be called again once per item before finishing it (drain protocol). */
class DrainService : public MockService {
public:
	itemProcessor_t createItemProcessor() override {
		auto pending = std::make_shared<workItem_t*>(nullptr);
		return [pending](workItem_t* item) -> bool {
			if (*pending) {
				workItem_t* p = *pending;
				for (unsigned i = 0; i < p->size(); ++i) p->resultBuffer()[i] = p->inputBuffer()[i] * *p->common();
				p->setProcessed();
				*pending = nullptr;
			}
			if (item) {
				*pending = item;
				return true;
			}
			return false;
		};
	}
};

class TimeOutService : public MockService {
public:
	itemProcessor_t createItemProcessor() override {
		return [](workItem_t*) -> bool { return false; };
	}
};

class ThrowingService : public MockService {
public:
	itemProcessor_t createItemProcessor() override {
		return [](workItem_t* item) -> bool {
			if (item) throw std::runtime_error("device failure in item processor");
			return false;
		};
	}
};

int main() {
	using request_t = Server<MockTypes>::request_t;
	/* construction / setService (Server_Test.cpp:30-80) */
	CHECK(error_of([] { Server<MockTypes> s(nullptr); }) == "Invalid service (nullptr).");
	CHECK(error_of([] { Server<MockTypes> s(std::make_shared<MockService>(false)); }) ==
			"Invalid service allocators (nullptr).");
	{
		Server<MockTypes> s(std::make_shared<MockService>());
		CHECK(error_of([&] { s.setService(nullptr); }) == "Invalid service (nullptr).");
		CHECK(error_of([&] { s.setItemSize(0); }) == "Item size must be greater than zero.");
		CHECK(error_of([&] { s.setItemSize(7); }).empty() && s.itemSize() == 7);
	}
	/* submit (Server_Test.cpp:82-127) */
	{
		Server<MockTypes> s(std::make_shared<MockService>());
		s.createWorkers(1);
		request_t r;
		CHECK(error_of([&] { s.submit(r); }) == "Invalid input buffer (nullptr).");
		std::vector<int> in(100000, 3), out(100000, 0);
		r.setDataAndSize(in.data(), in.size());
		r.setCommon(2);
		CHECK(error_of([&] { s.submit(r); r.setDataAndSize(in.data(), in.size()); s.submit(r); }) ==
				"Request has already been submitted.");
		s.wait(r, out.data());
		CHECK(out[0] == 6 && out[99999] == 6);
		for (int i = 0; i < 10; ++i) {
			r.setDataAndSize(in.data(), 0);
			CHECK(error_of([&] { s.submit(r); s.wait(r, out.data()); }).empty());
		}
	}
	/* wait (Server_Test.cpp:129-182) */
	{
		Server<MockTypes> s(std::make_shared<MockService>());
		s.createWorkers(1);
		int in[1] = {5}, out[1] = {0};
		request_t r(in, 1, 3);
		s.submit(r);
		request_t other;
		CHECK(error_of([&] { s.wait(other, out); }) ==
				"Either request has not been submitted or clientBuffer invalid (nullptr).");
		CHECK(error_of([&] { s.wait(r, nullptr); }) ==
				"Either request has not been submitted or clientBuffer invalid (nullptr).");
		s.wait(r, out);
		CHECK(out[0] == 15);
		Server<MockTypes> st(std::make_shared<TimeOutService>());
		st.createWorkers(1);
		st.setWaitTime(10);
		request_t rt(in, 1, 1);
		st.submit(rt);
		CHECK(error_of([&] { st.wait(rt, out); }) == "Request takes too long to finish for unknown reasons");
	}
	/* a failing item processor surfaces in wait, the worker survives */
	{
		Server<MockTypes> s(std::make_shared<ThrowingService>());
		s.createWorkers(2);
		std::vector<int> in(50, 1), out(50, 0);
		request_t r(in.data(), in.size(), 1);
		s.submit(r);
		CHECK(error_of([&] { s.wait(r, out.data()); }) == "device failure in item processor");
		request_t r2(in.data(), in.size(), 1);
		s.submit(r2);
		CHECK(!error_of([&] { s.wait(r2, out.data()); }).empty());
	}
	/* split / dispatch / gather sweep (Server_Test.cpp:208-277) */
	for (unsigned workers : {1u, 2u, 3u, 4u})
		for (size_t item : {size_t(1), size_t(7), size_t(100), size_t(1000)})
			for (size_t n : {size_t(1), size_t(10), size_t(999), size_t(100000)}) {
				if (item == 1 && n == 100000) continue;
				for (int drain = 0; drain < 2; ++drain) {
					Server<MockTypes> s(drain ? std::make_shared<DrainService>() : std::make_shared<MockService>());
					s.createWorkers(workers);
					s.setItemSize(item);
					std::vector<int> in(n), out(n, -1);
					for (size_t i = 0; i < n; ++i) in[i] = (int)(i % 1000) - 500;
					request_t r(in.data(), n, 3);
					s.submit(r);
					s.wait(r, out.data());
					bool ok = true;
					for (size_t i = 0; i < n; ++i) ok &= out[i] == 3 * in[i];
					CHECK(ok);
				}
			}
	/* several requests in flight at once */
	{
		Server<MockTypes> s(std::make_shared<MockService>());
		s.createWorkers(3);
		s.setItemSize(13);
		std::vector<std::vector<int>> ins(8), outs(8);
		std::vector<request_t> reqs(8);
		for (int k = 0; k < 8; ++k) {
			ins[k].assign(1000 + 37 * k, k + 1);
			outs[k].assign(ins[k].size(), 0);
			reqs[k] = request_t(ins[k].data(), ins[k].size(), k);
			s.submit(reqs[k]);
		}
		for (int k = 7; k >= 0; --k) {
			s.wait(reqs[k], outs[k].data());
			CHECK(outs[k].front() == k * (k + 1) && outs[k].back() == k * (k + 1));
		}
	}
	if (failures) {
		std::fprintf(stderr, "%d failures\n", failures);
		return 1;
	}
	std::printf("OK\n");
	return 0;
}
