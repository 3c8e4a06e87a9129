// tc_mma_rate.cu -- rate of a bare tcgen05.mma stream (kind::f16, BF16 in,
// FP32 accumulate, M=128, K=16) with both operands resident in shared memory,
// one CTA per SM: N in {64,128,256}; the A start row aligned (mode 0), shifted
// by 3 rows (mode 1), or cycling through the nine 3x3 tap shifts of the L3
// layout (mode 2); the B start row (N rows) cycling through the nine tap
// shifts (mode 3, the conv kernels' case) or through nine multiples of 8
// rows (mode 4); mode 5 = mode 3 plus, every 4 MMAs, the per-stage handshake
// of the conv kernels (tcgen05.commit to an mbarrier, an mbarrier wait that
// is already satisfied, tcgen05.fence::after_thread_sync).  Build and run on
// a GB300:
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 \
//        -o tc_mma_rate leela_gb300/microbench/tc_mma_rate.cu && ./tc_mma_rate
#include <cstdio>
#include <vector>
#include "../csrc/lg_common.cuh"
void lg_set_error(const char *fmt, ...) {}
using namespace lg;
using namespace lg::ptx;

__device__ __forceinline__ uint32_t idesc_n(int N) { return idesc_bf16(128, N); }

// MODE: 0 = aligned, 1 = A shifted by 3 rows, 2 = A cycling 9 tap shifts,
// 3 = B cycling 9 tap shifts, 4 = B cycling 9 multiples of 8 rows, 5 = 3 plus
// the per-stage handshake.  The 36
// (tap, K step) descriptors of one round are compile-time offsets of two base
// descriptors (the start-address field is addr >> 4 in the low 14 bits and
// never carries), so the one issuing thread spends a few instructions per MMA.
template <int N, int MODE>
__global__ void __launch_bounds__(128, 1) bench(int rounds, unsigned long long *cycles, int *err) {
    extern __shared__ __align__(1024) uint8_t raw[];
    uint8_t *sm = (uint8_t *)(((uintptr_t)raw + 1023) & ~(uintptr_t)1023);
    uint8_t *A = sm;                 // 256 rows x 128 B
    uint8_t *Bm = sm + 256 * 128;    // 256 + 64 rows x 128 B
    __shared__ uint64_t bar, bar2[4], bar3;
    __shared__ uint32_t tb;
    int tid = threadIdx.x, warp = tid / 32;
    for (int i = tid; i < 576 * 128 / 16; i += 128) reinterpret_cast<uint4 *>(sm)[i] = make_uint4(0, 0, 0, 0);
    fence_proxy_async();
    if (tid == 0) {
        mbar_init(&bar, 1);
        for (int i = 0; i < 4; ++i) mbar_init(&bar2[i], (1 << 20) - 1);  // never completes: commits only count
        mbar_init(&bar3, 1);
        fence_mbar_init();
        mbar_arrive(&bar3);  // phase 0 complete: waits on it return at once
    }
    if (warp == 0) tmem_alloc(&tb, 256);
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
        constexpr uint32_t id = idesc_bf16(128, N);
        const uint64_t a0 = sdesc_sw128(smem_u32(A)), b0 = sdesc_sw128(smem_u32(Bm));
        unsigned long long t0 = clock64();
        for (int r = 0; r < rounds; ++r) {
#pragma unroll
            for (int u = 0; u < 36; ++u) {
                const int t9 = u / 4, kk = u % 4;
                const int tap = 3 + (t9 / 3) * 20 + t9 % 3;  // the 3x3 tap shifts 3,4,5,23,..,45 (L3 pitch 20)
                const int ra = MODE == 1 ? 3 : (MODE == 2 ? tap : 0);
                const int rb = (MODE == 3 || MODE == 5) ? tap : (MODE == 4 ? 8 * t9 : 0);
                mma_bf16(tb, a0 + (uint64_t)((ra * 128 + kk * 32) >> 4), b0 + (uint64_t)((rb * 128 + kk * 32) >> 4), id,
                         (r > 0 || u > 0) ? 1u : 0u);
                if (MODE >= 5 && kk == 3) {
                    mma_commit(&bar2[t9 & 3]);
                    if (!mbar_wait(&bar3, 0, 1u << 20)) atomicExch(err, 2);
                    tc_fence_after();
                }
            }
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

template <int N, int MODE>
void run(int sms, int smem, int rounds, unsigned long long *dc, int *de) {
    cudaFuncSetAttribute(bench<N, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    std::vector<unsigned long long> h(sms);
    for (int grid : {1, sms}) {
        cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
        cudaEventRecord(a);
        bench<N, MODE><<<grid, 128, smem>>>(rounds, dc, de);
        cudaEventRecord(b);
        cudaError_t e = cudaEventSynchronize(b);
        float ms; cudaEventElapsedTime(&ms, a, b);
        cudaMemcpy(h.data(), dc, grid * 8, cudaMemcpyDeviceToHost);
        unsigned long long mx = 0; for (int i = 0; i < grid; ++i) mx = h[i] > mx ? h[i] : mx;
        double macs = 128.0 * N * 16 * 36 * rounds;
        printf("N=%3d mode=%d grid=%3d: %8llu clk  %.0f MAC/clk/SM  %.1f TFLOP/s total (%.3f ms) %s\n", N, MODE, grid, mx,
               macs / mx, 2 * macs * grid / (ms * 1e-3) / 1e12, ms, cudaGetErrorString(e));
    }
}

int main() {
    int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    unsigned long long *dc; int *de;
    cudaMalloc(&dc, sms * 8); cudaMalloc(&de, 4); cudaMemset(de, 0, 4);
    const int smem = 1024 + 576 * 128, rounds = 114;  // 4104 MMAs per CTA
    run<64, 0>(sms, smem, rounds, dc, de);
    run<128, 0>(sms, smem, rounds, dc, de);
    run<256, 0>(sms, smem, rounds, dc, de);
    run<256, 1>(sms, smem, rounds, dc, de);
    run<256, 2>(sms, smem, rounds, dc, de);
    run<256, 3>(sms, smem, rounds, dc, de);
    run<256, 4>(sms, smem, rounds, dc, de);
    run<128, 3>(sms, smem, rounds, dc, de);
    run<256, 5>(sms, smem, rounds, dc, de);
    int he; cudaMemcpy(&he, de, 4, cudaMemcpyDeviceToHost);
    printf("err=%d\n", he);
    return 0;
}
