// tc_mma_rate.cu -- rate of a bare tcgen05.mma stream (kind::f16, BF16 in,
// FP32 accumulate, M=128, K=16) with both operands resident in shared memory,
// one CTA per SM: N in {64,128,256}; the A start row aligned (mode 0), shifted
// by 3 rows (mode 1), or cycling through the nine 3x3 tap shifts of the L3
// layout (mode 2).  Build and run on a GB300:
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 \
//        -o tc_mma_rate leela_gb300/microbench/tc_mma_rate.cu && ./tc_mma_rate
#include <cstdio>
#include <vector>
#include "../csrc/lg_common.cuh"
void lg_set_error(const char *fmt, ...) {}
using namespace lg;
using namespace lg::ptx;

__device__ __forceinline__ uint32_t idesc_n(int N) { return idesc_bf16(128, N); }

// mode: 0 = aligned A, 1 = A shifted by 3 rows, 2 = A cycling 9 tap shifts
template <int N>
__global__ void __launch_bounds__(128, 1) bench(int iters, int mode, unsigned long long *cycles, int *err) {
    extern __shared__ __align__(1024) uint8_t raw[];
    uint8_t *sm = (uint8_t *)(((uintptr_t)raw + 1023) & ~(uintptr_t)1023);
    uint8_t *A = sm;                 // 256 rows x 128 B
    uint8_t *Bm = sm + 256 * 128;    // 256 rows x 128 B
    __shared__ uint64_t bar;
    __shared__ uint32_t tb;
    int tid = threadIdx.x, warp = tid / 32;
    for (int i = tid; i < 512 * 128 / 16; i += 128) reinterpret_cast<uint4 *>(sm)[i] = make_uint4(0, 0, 0, 0);
    fence_proxy_async();
    if (tid == 0) { mbar_init(&bar, 1); fence_mbar_init(); }
    if (warp == 0) tmem_alloc(&tb, 256);
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
        const int shifts[9] = {3, 4, 5, 23, 24, 25, 43, 44, 45};
        uint32_t id = idesc_n(N);
        unsigned long long t0 = clock64();
        for (int i = 0; i < iters; ++i) {
            int r = mode == 0 ? 0 : (mode == 1 ? 3 : shifts[(i >> 2) % 9]);
            uint64_t ad = sdesc_sw128(smem_u32(A + r * 128 + (i & 3) * 32));
            uint64_t bd = sdesc_sw128(smem_u32(Bm + (i & 3) * 32));
            mma_bf16(tb, ad, bd, id, i > 0);
        }
        mma_commit(&bar);
        if (!mbar_wait(&bar, 0, 1u << 28)) atomicExch(err, 1);
        unsigned long long t1 = clock64();
        cycles[blockIdx.x] = t1 - t0;
    }
    __syncthreads();
    tc_fence_after();
    if (warp == 0) { tmem_dealloc(tb, 256); tmem_relinquish(); }
}

int main() {
    int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    unsigned long long *dc; int *de;
    cudaMalloc(&dc, sms * 8); cudaMalloc(&de, 4); cudaMemset(de, 0, 4);
    int smem = 1024 + 512 * 128;
    cudaFuncSetAttribute(bench<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(bench<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(bench<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    std::vector<unsigned long long> h(sms);
    const int iters = 4096;
    for (int n : {64, 128, 256})
        for (int mode = 0; mode < 3; ++mode)
            for (int grid : {1, sms}) {
                cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
                cudaEventRecord(a);
                if (n == 64) bench<64><<<grid, 128, smem>>>(iters, mode, dc, de);
                if (n == 128) bench<128><<<grid, 128, smem>>>(iters, mode, dc, de);
                if (n == 256) bench<256><<<grid, 128, smem>>>(iters, mode, dc, de);
                cudaEventRecord(b);
                cudaError_t e = cudaEventSynchronize(b);
                float ms; cudaEventElapsedTime(&ms, a, b);
                cudaMemcpy(h.data(), dc, grid * 8, cudaMemcpyDeviceToHost);
                unsigned long long mx = 0; for (int i = 0; i < grid; ++i) mx = h[i] > mx ? h[i] : mx;
                double macs = 128.0 * n * 16 * iters;
                printf("N=%3d mode=%d grid=%3d: %8llu clk  %.0f MAC/clk/SM  %.1f TFLOP/s total (%.3f ms) %s\n", n, mode, grid, mx,
                       macs / mx, 2 * macs * grid / (ms * 1e-3) / 1e12, ms, cudaGetErrorString(e));
            }
    int he; cudaMemcpy(&he, de, 4, cudaMemcpyDeviceToHost);
    printf("err=%d\n", he);
    return 0;
}
