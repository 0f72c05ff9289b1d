/*
 * pose_order.cu -- spatial visiting order of a batch of poses.
 *
 * The warps resident at any moment (a few thousand poses) touch the grid
 * around their ligand positions.  In submission order those poses are spread
 * over the whole docking shell, so the gathered octets come from the whole
 * grid (hundreds of MB, far beyond the L2).  Visiting poses grouped by pair
 * and, within a pair, in Morton order of their translation keeps the resident
 * set spatially compact and its grid working set L2-sized.  Only the visiting
 * order changes: every pose still writes its own output slot, so results are
 * identical to unordered runs.
 */
#include <cub/device/device_radix_sort.cuh>

#include "gba_context.h"

namespace gba {

namespace {

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
	v &= 0x3ffu;
	v = (v | (v << 16)) & 0x030000ffu;
	v = (v | (v << 8)) & 0x0300f00fu;
	v = (v | (v << 4)) & 0x030c30c3u;
	v = (v | (v << 2)) & 0x09249249u;
	return v;
}

/* key = pair << 32 | Morton(translation in the pair's outer-grid box) */
__global__ void order_keys_kernel(const float* __restrict__ dofs, size_t stride_floats, size_t n,
		DevIntrpl box, const RigidModel* __restrict__ models, const uint32_t* __restrict__ pair_of,
		unsigned long long* __restrict__ keys, uint32_t* __restrict__ idx) {
	const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= n) return;
	uint32_t pair = 0;
	const DevIntrpl* b = &box;
	if (pair_of) {
		pair = __ldg(&pair_of[p]);
		b = &models[pair].grid.outer;
	}
	const float* d = dofs + p * stride_floats;
	uint32_t q[3];
#pragma unroll
	for (int a = 0; a < 3; ++a) {
		const float ext = fmaxf(b->maxDim[a] - b->pos[a], 1e-3f);
		float t = (__ldg(d + a) - b->pos[a]) * (1024.f / ext);
		t = fminf(fmaxf(t, 0.f), 1023.f);      /* NaN -> 0 */
		q[a] = (uint32_t)t;
	}
	const uint32_t m = spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2);
	keys[p] = ((unsigned long long)pair << 32) | m;
	idx[p] = (uint32_t)p;
}

int key_bits(size_t npairs) {
	int b = 30;
	if (npairs > 1) {
		b = 32;
		size_t v = npairs - 1;
		while (v) { ++b; v >>= 1; }
	}
	return b;
}

/* Sorts with buffers from `get(slot, bytes)`; returns the ordered indices. */
template <typename Get>
const uint32_t* sort_order(const void* dofs, size_t stride_floats, size_t n, const DevIntrpl& box,
		const RigidModel* models, const uint32_t* pair_of, size_t npairs, cudaStream_t s, Get get) {
	unsigned long long* k0 = (unsigned long long*)get(0, n * 8);
	unsigned long long* k1 = (unsigned long long*)get(1, n * 8);
	uint32_t* i0 = (uint32_t*)get(2, n * 4);
	uint32_t* i1 = (uint32_t*)get(3, n * 4);
	order_keys_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>((const float*)dofs, stride_floats,
			n, box, models, pair_of, k0, i0);
	check_cuda(cudaGetLastError(), "pose order: keys");
	cub::DoubleBuffer<unsigned long long> kb(k0, k1);
	cub::DoubleBuffer<uint32_t> ib(i0, i1);
	const int end_bit = key_bits(npairs);
	size_t tmp = 0;
	check_cuda(cub::DeviceRadixSort::SortPairs(nullptr, tmp, kb, ib, (int)n, 0, end_bit, s),
			"pose order: sort size");
	void* t = get(4, tmp);
	check_cuda(cub::DeviceRadixSort::SortPairs(t, tmp, kb, ib, (int)n, 0, end_bit, s), "pose order: sort");
	return ib.Current();
}

}  // namespace

/* Order for one launch; scratch from the stream-ordered allocator, released
 * on `s` by `scratch`'s destructor after the kernels that read it. */
const uint32_t* Context::pose_order(const void* dofs, size_t stride_floats, size_t n,
		const DevIntrpl& box, cudaStream_t s, StreamScratch& scratch) {
	if (!order_enabled || n < kOrderMinPoses || n > 0x7fffffffull) return nullptr;
	return sort_order(dofs, stride_floats, n, box, nullptr, nullptr, 1, s,
			[&](int, size_t bytes) { return scratch.get(bytes, s); });
}

/* Order kept in context buffers (stable addresses for the cached minimizer
 * graph); the caller holds stage_mu. */
const uint32_t* Context::pose_order_persistent(const void* dofs, size_t stride_floats, size_t n,
		const DevIntrpl& box, const RigidModel* models, const uint32_t* pair_of, size_t npairs,
		cudaStream_t s) {
	if (!order_enabled || n < kOrderMinPoses || n > 0x7fffffffull) return nullptr;
	return sort_order(dofs, stride_floats, n, box, models, pair_of, npairs, s,
			[&](int slot, size_t bytes) {
				DevBuffer& b = order_buf[slot];
				if (b.bytes < bytes) b.alloc(bytes + bytes / 4 + 256);
				return b.ptr;
			});
}

/* Order computed in caller-provided device memory [buf, buf + cap) (256-byte
 * aligned carving); ApiError when the keys, indices and sort scratch do not fit. */
const uint32_t* pose_order_in(const void* dofs, size_t stride_floats, size_t n, const DevIntrpl& box,
		void* buf, size_t cap, cudaStream_t s) {
	size_t used = 0;
	return sort_order(dofs, stride_floats, n, box, nullptr, nullptr, 1, s, [&](int, size_t bytes) {
		const size_t at = (used + 255) & ~(size_t)255;
		if (at + bytes > cap)
			throw ApiError(GBA_ERR_INVALID_ARGUMENT, "visiting order: " + std::to_string(at + bytes) +
					" bytes of scratch needed, " + std::to_string(cap) + " available");
		used = at + bytes;
		return (void*)((char*)buf + at);
	});
}

void* StreamScratch::get(size_t bytes, cudaStream_t s) {
	void* p = nullptr;
	check_cuda(cudaMallocAsync(&p, bytes ? bytes : 16, s), "cudaMallocAsync");
	ptrs.push_back(p);
	stream = s;
	return p;
}

StreamScratch::~StreamScratch() {
	for (void* p : ptrs) cudaFreeAsync(p, stream);
}

}  // namespace gba
