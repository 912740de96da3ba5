// Test-only kernel: curand's Philox4x32-10 block function on a list of
// (counter, key) pairs, to pin the project's Philox (device and oracle) to
// the CUDA toolkit's implementation.  Built by tests/test_gpu_parity.py.
#include <curand_kernel.h>
#include <cstdint>

__global__ void curand_philox_kernel(const uint4 *ctr, const uint2 *key, uint4 *out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = curand_Philox4x32_10(ctr[i], key[i]);
}

extern "C" int curand_philox_batch(const uint32_t *ctr, const uint32_t *key, uint32_t *out, int n) {
    uint4 *dc = nullptr, *dout = nullptr;
    uint2 *dk = nullptr;
    if (cudaMalloc(&dc, n * sizeof(uint4)) != cudaSuccess) return 1;
    cudaMalloc(&dk, n * sizeof(uint2));
    cudaMalloc(&dout, n * sizeof(uint4));
    cudaMemcpy(dc, ctr, n * sizeof(uint4), cudaMemcpyHostToDevice);
    cudaMemcpy(dk, key, n * sizeof(uint2), cudaMemcpyHostToDevice);
    curand_philox_kernel<<<(n + 127) / 128, 128>>>(dc, dk, dout, n);
    const cudaError_t e = cudaMemcpy(out, dout, n * sizeof(uint4), cudaMemcpyDeviceToHost);
    cudaFree(dc);
    cudaFree(dk);
    cudaFree(dout);
    return e == cudaSuccess ? 0 : 2;
}
