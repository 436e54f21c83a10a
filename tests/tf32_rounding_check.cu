// Compares the engine's TF32 rounding (qcs::tc::tf32_rna, integer form) with cvt.rna.tf32.f32 on every
// 32-bit pattern whose value is finite; prints the number of differing values below the overflow
// threshold and the number at or above it.  Built and run by tests/test_gpu_tf32_rounding.py.
#include <cstdio>
#include <cuda_runtime.h>

#include "tcgen05.cuh"

__device__ unsigned long long g_diff[2];

__global__ void check(unsigned long long begin, unsigned long long count) {
	unsigned long long mine[2] = {0, 0};
	for (unsigned long long i = blockIdx.x * 256ull + threadIdx.x; i < count; i += gridDim.x * 256ull) {
		const uint32_t u = static_cast<uint32_t>(begin + i);
		if ((u & 0x7F800000u) == 0x7F800000u) continue;  // Inf and NaN
		const float x = __uint_as_float(u);
		uint32_t ref;
		asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(ref) : "f"(x));
		const uint32_t got = __float_as_uint(qcs::tc::tf32_rna(x));
		if (got != ref) ++mine[(u & 0x7FFFFFFFu) >= 0x7F7FF000u ? 1 : 0];
	}
	if (mine[0]) atomicAdd(&g_diff[0], mine[0]);
	if (mine[1]) atomicAdd(&g_diff[1], mine[1]);
}

int main() {
	const unsigned long long total = 1ull << 32, chunk = 1ull << 30;
	for (unsigned long long b = 0; b < total; b += chunk) check<<<1024, 256>>>(b, chunk);
	unsigned long long diff[2] = {0, 0};
	cudaError_t e = cudaMemcpyFromSymbol(diff, g_diff, sizeof(diff));
	if (e != cudaSuccess) {
		std::printf("cuda error %s\n", cudaGetErrorString(e));
		return 1;
	}
	std::printf("differ_below_overflow %llu differ_at_overflow %llu\n", diff[0], diff[1]);
	return 0;
}
