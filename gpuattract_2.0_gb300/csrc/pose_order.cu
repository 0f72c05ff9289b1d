/*
 * pose_order.cu -- spatial visiting order of a batch of poses.
 *
 * The warps resident at any moment (a few thousand poses) touch the grid
 * around their ligand positions.  In submission order those poses are spread
 * over the whole docking shell, so the gathered octets come from the whole
 * grid (hundreds of MB, far beyond the L2).  Visiting poses grouped by pair
 * and, within a pair, by translation keeps the resident set spatially compact
 * and its grid working set smaller.  One pair's scoring launch groups its
 * poses by 32^3 translation cells (a counting sort: cheap on the host, which
 * otherwise leaves the GPU idle before the launch); multi-pair minimizer
 * batches sort (pair, Morton key) with a radix sort.  Only the visiting order
 * changes: every pose still writes its own output slot, so results are
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

constexpr int kMortonBits = 8;   /* per axis: 256 cells across the outer-grid box */

/* key = rank(pair) << 24 | Morton(translation in the pair's outer-grid box);
 * rank = pair_rank[pair] when given, else the pair index */
template <typename K>
__global__ void order_keys_kernel(const float* __restrict__ dofs, size_t stride_floats, size_t n,
		DevIntrpl box, const RigidModel* __restrict__ models, const uint32_t* __restrict__ pair_of,
		const uint32_t* __restrict__ pair_rank, K* __restrict__ keys, uint32_t* __restrict__ idx) {
	const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= n) return;
	uint32_t pair = 0;
	const DevIntrpl* b = &box;
	if (pair_of) {
		pair = __ldg(&pair_of[p]);
		b = &models[pair].grid.outer;
	}
	const uint32_t rank = pair_rank ? __ldg(&pair_rank[pair]) : pair;
	const float* d = dofs + p * stride_floats;
	constexpr float cells = (float)(1 << kMortonBits);
	uint32_t q[3];
#pragma unroll
	for (int a = 0; a < 3; ++a) {
		const float ext = fmaxf(b->maxDim[a] - b->pos[a], 1e-3f);
		float t = (__ldg(d + a) - b->pos[a]) * (cells / ext);
		t = fminf(fmaxf(t, 0.f), cells - 1.f);      /* NaN -> 0 */
		q[a] = (uint32_t)t;
	}
	const uint32_t m = spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2);
	keys[p] = ((K)rank << (3 * kMortonBits)) | m;
	idx[p] = (uint32_t)p;
}

int key_bits(size_t npairs) {
	int b = 3 * kMortonBits;
	for (size_t v = npairs > 1 ? npairs - 1 : 0; v; v >>= 1) ++b;
	return b;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

/* Keys, indices (double-buffered) and the radix-sort scratch in one block
 * from `get(bytes)`; returns the ordered indices. */
template <typename K, typename Get>
const uint32_t* sort_keys(const void* dofs, size_t stride_floats, size_t n, const DevIntrpl& box,
		const RigidModel* models, const uint32_t* pair_of, const uint32_t* pair_rank, int end_bit,
		cudaStream_t s, Get get) {
	cub::DoubleBuffer<K> kb(nullptr, nullptr);
	cub::DoubleBuffer<uint32_t> ib(nullptr, nullptr);
	size_t tmp = 0;
	check_cuda(cub::DeviceRadixSort::SortPairs(nullptr, tmp, kb, ib, (int)n, 0, end_bit, s),
			"pose order: sort size");
	const size_t kbytes = align256(n * sizeof(K)), ibytes = align256(n * sizeof(uint32_t));
	char* base = (char*)get(2 * kbytes + 2 * ibytes + align256(tmp));
	K* k0 = (K*)base;
	K* k1 = (K*)(base + kbytes);
	uint32_t* i0 = (uint32_t*)(base + 2 * kbytes);
	uint32_t* i1 = (uint32_t*)(base + 2 * kbytes + ibytes);
	void* t = base + 2 * kbytes + 2 * ibytes;
	order_keys_kernel<K><<<(unsigned)((n + 255) / 256), 256, 0, s>>>((const float*)dofs, stride_floats,
			n, box, models, pair_of, pair_rank, k0, i0);
	check_cuda(cudaGetLastError(), "pose order: keys");
	kb = cub::DoubleBuffer<K>(k0, k1);
	ib = cub::DoubleBuffer<uint32_t>(i0, i1);
	check_cuda(cub::DeviceRadixSort::SortPairs(t, tmp, kb, ib, (int)n, 0, end_bit, s), "pose order: sort");
	return ib.Current();
}

constexpr int kBucketBits = 5;                       /* per axis: 32^3 translation cells */
constexpr int kBuckets = 1 << (3 * kBucketBits);

/* Bucket (Morton cell of the translation in the outer-grid box) of pose p,
 * and the pose's rank inside it. */
__global__ void bucket_keys_kernel(const float* __restrict__ dofs, size_t stride_floats, size_t n, DevIntrpl box,
		uint32_t* __restrict__ count, uint32_t* __restrict__ bucket, uint32_t* __restrict__ rank) {
	const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= n) return;
	const float* d = dofs + p * stride_floats;
	constexpr float cells = (float)(1 << kBucketBits);
	uint32_t q[3];
#pragma unroll
	for (int a = 0; a < 3; ++a) {
		const float ext = fmaxf(box.maxDim[a] - box.pos[a], 1e-3f);
		float t = (__ldg(d + a) - box.pos[a]) * (cells / ext);
		t = fminf(fmaxf(t, 0.f), cells - 1.f);      /* NaN -> 0 */
		q[a] = (uint32_t)t;
	}
	const uint32_t b = spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2);
	bucket[p] = b;
	rank[p] = atomicAdd(&count[b], 1u);
}

/* Exclusive prefix sum of the kBuckets counts, one 1024-thread block. */
__global__ void __launch_bounds__(1024) bucket_scan_kernel(uint32_t* __restrict__ count) {
	constexpr int per = kBuckets / 1024;
	__shared__ uint32_t warp_tot[32];
	const int t = threadIdx.x, lane = t & 31, w = t >> 5;
	uint32_t v[per];
	uint32_t sum = 0;
#pragma unroll
	for (int k = 0; k < per; ++k) { v[k] = count[t * per + k]; sum += v[k]; }
	uint32_t incl = sum;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const uint32_t x = __shfl_up_sync(0xffffffffu, incl, o);
		if (lane >= o) incl += x;
	}
	if (lane == 31) warp_tot[w] = incl;
	__syncthreads();
	if (w == 0) {
		uint32_t x = warp_tot[lane], xi = x;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const uint32_t y = __shfl_up_sync(0xffffffffu, xi, o);
			if (lane >= o) xi += y;
		}
		warp_tot[lane] = xi - x;
	}
	__syncthreads();
	uint32_t run = warp_tot[w] + incl - sum;
#pragma unroll
	for (int k = 0; k < per; ++k) { count[t * per + k] = run; run += v[k]; }
}

__global__ void bucket_scatter_kernel(size_t n, const uint32_t* __restrict__ start,
		const uint32_t* __restrict__ bucket, const uint32_t* __restrict__ rank, uint32_t* __restrict__ order) {
	const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= n) return;
	order[start[bucket[p]] + rank[p]] = (uint32_t)p;
}

/* Visiting order of one pair's poses grouped by translation cell: a counting
 * sort (one memset, three small kernels) whose host cost stays far below a
 * radix sort's; poses of a cell keep no particular order. */
template <typename Get>
const uint32_t* bucket_order(const void* dofs, size_t stride_floats, size_t n, const DevIntrpl& box,
		cudaStream_t s, Get get) {
	const size_t cbytes = align256(kBuckets * sizeof(uint32_t)), nbytes = align256(n * sizeof(uint32_t));
	char* base = (char*)get(cbytes + 3 * nbytes);
	uint32_t* count = (uint32_t*)base;
	uint32_t* bucket = (uint32_t*)(base + cbytes);
	uint32_t* rank = (uint32_t*)(base + cbytes + nbytes);
	uint32_t* order = (uint32_t*)(base + cbytes + 2 * nbytes);
	check_cuda(cudaMemsetAsync(count, 0, kBuckets * sizeof(uint32_t), s), "pose order: clear");
	const unsigned blocks = (unsigned)((n + 255) / 256);
	bucket_keys_kernel<<<blocks, 256, 0, s>>>((const float*)dofs, stride_floats, n, box, count, bucket, rank);
	bucket_scan_kernel<<<1, 1024, 0, s>>>(count);
	bucket_scatter_kernel<<<blocks, 256, 0, s>>>(n, count, bucket, rank, order);
	check_cuda(cudaGetLastError(), "pose order: buckets");
	return order;
}

/* 32-bit keys while they fit (up to 256 pairs), else 64-bit. */
template <typename Get>
const uint32_t* sort_order(const void* dofs, size_t stride_floats, size_t n, const DevIntrpl& box,
		const RigidModel* models, const uint32_t* pair_of, const uint32_t* pair_rank, size_t npairs,
		cudaStream_t s, Get get) {
	const int end_bit = key_bits(npairs);
	if (end_bit <= 32)
		return sort_keys<uint32_t>(dofs, stride_floats, n, box, models, pair_of, pair_rank, end_bit, s, get);
	return sort_keys<unsigned long long>(dofs, stride_floats, n, box, models, pair_of, pair_rank, end_bit, s,
			get);
}

}  // namespace

/* Order for one launch; scratch from the stream-ordered allocator, released
 * on `s` by `scratch`'s destructor after the kernels that read it. */
const uint32_t* Context::pose_order(const void* dofs, size_t stride_floats, size_t n,
		const DevIntrpl& box, cudaStream_t s, StreamScratch& scratch) {
	if (!order_enabled || n < kOrderMinPoses || n > 0x7fffffffull) return nullptr;
	return bucket_order(dofs, stride_floats, n, box, s, [&](size_t bytes) { return scratch.get(bytes, s); });
}

/* Order kept in context buffers (stable addresses for the cached minimizer
 * graph); the caller holds stage_mu. */
const uint32_t* Context::pose_order_persistent(const void* dofs, size_t stride_floats, size_t n,
		const DevIntrpl& box, const RigidModel* models, const uint32_t* pair_of, const uint32_t* pair_rank,
		size_t npairs, cudaStream_t s) {
	if (!order_enabled || n < kOrderMinPoses || n > 0x7fffffffull) return nullptr;
	return sort_order(dofs, stride_floats, n, box, models, pair_of, pair_rank, npairs, s,
			[&](size_t bytes) {
				DevBuffer& b = order_buf;
				if (b.bytes < bytes) b.alloc(bytes + bytes / 4 + 256);
				return b.ptr;
			});
}

/* Order computed in caller-provided device memory [buf, buf + cap) (256-byte
 * aligned carving); ApiError when the keys, indices and sort scratch do not fit. */
const uint32_t* pose_order_in(const void* dofs, size_t stride_floats, size_t n, const DevIntrpl& box,
		void* buf, size_t cap, cudaStream_t s) {
	size_t used = 0;
	return bucket_order(dofs, stride_floats, n, box, s, [&](size_t bytes) {
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
	note_allocation();
	if (pool)
		check_cuda(cudaMallocFromPoolAsync(&p, bytes ? bytes : 16, pool, s), "cudaMallocFromPoolAsync");
	else
		check_cuda(cudaMallocAsync(&p, bytes ? bytes : 16, s), "cudaMallocAsync");
	ptrs.push_back(p);
	stream = s;
	return p;
}

StreamScratch::~StreamScratch() {
	for (void* p : ptrs) cudaFreeAsync(p, stream);
}

}  // namespace gba
