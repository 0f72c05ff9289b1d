/* Device harness: the VA13 machine's warp form (VA13::provide_w with
 * VaWarp, element j on lane j) stepped by one warp on the GPU, on the
 * objectives of va13_objectives.h (lane 0 evaluates them; they give the same
 * bits on the host), for an exact comparison with the host machine's trace
 * (va13_trace.cpp, va13_trace_form). */
#include <cuda_runtime.h>

#include "../../gpuattract_2.0_gb300/csrc/va13.cuh"
#include "va13_objectives.h"

namespace {

constexpr int kMaxN = 31;

/* one warp; out: cap rows of (point, f); count: rows written */
__global__ void trace_kernel(int n, const double* x0, int ivmax, double* out, int cap, int nan_eval, int kind,
		int* count) {
	__shared__ gba::VA13<kMaxN> va;
	__shared__ double f_s, g_s[kMaxN];
	const int lane = threadIdx.x & 31;
	if (lane == 0) va.start(x0, n, ivmax);
	__syncwarp();
	int k = 0;
	/* the machine ends within ivmax + 1 evaluations; cap bounds the loop
	 * whatever it does */
	while (k < cap) {
		if (__shfl_sync(0xffffffffu, (int)va.done(), 0)) break;
		if (lane == 0) {
			const double* s = va.point();
			double g[kMaxN];
			const double f = va13_exact_objective(kind, n, s, g);
			if (k == nan_eval) g[0] = __longlong_as_double(0x7ff8000000000000ll);
			for (int i = 0; i < n; ++i) out[(size_t)k * (n + 1) + i] = s[i];
			out[(size_t)k * (n + 1) + n] = f;
			f_s = f;
			for (int i = 0; i < n; ++i) g_s[i] = g[i];
		}
		__syncwarp();
		++k;
		const double f = f_s;
		const double gl = lane >= 1 && lane <= n ? g_s[lane - 1] : 0.0;
		/* its first __syncwarp orders these reads before lane 0's next writes */
		va.provide_w(f, [&](int) { return gl; }, gba::VaWarp{lane});
	}
	if (lane == 0) *count = k;
}

}  // namespace

/* Returns the number of trace rows (at most cap), or -1 on bad arguments or a
 * CUDA error. */
extern "C" int va13_device_trace(int n, const double* x0, int ivmax, double* out, int cap, int nan_eval,
		int kind) {
	if (n < 1 || n > kMaxN || cap < 1 || ivmax < 0 || !va13_exact_kind(kind)) return -1;
	double *dx = nullptr, *dout = nullptr;
	int* dcount = nullptr;
	int count = -1;
	const size_t out_bytes = (size_t)cap * (n + 1) * sizeof(double);
	bool ok = cudaMalloc(&dx, n * sizeof(double)) == cudaSuccess && cudaMalloc(&dout, out_bytes) == cudaSuccess &&
	          cudaMalloc(&dcount, sizeof(int)) == cudaSuccess &&
	          cudaMemcpy(dx, x0, n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
	          cudaMemset(dout, 0, out_bytes) == cudaSuccess;
	if (ok) {
		trace_kernel<<<1, 32>>>(n, dx, ivmax, dout, cap, nan_eval, kind, dcount);
		ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess &&
		     cudaMemcpy(&count, dcount, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess &&
		     cudaMemcpy(out, dout, out_bytes, cudaMemcpyDeviceToHost) == cudaSuccess;
	}
	cudaFree(dx);
	cudaFree(dout);
	cudaFree(dcount);
	return ok ? count : -1;
}
