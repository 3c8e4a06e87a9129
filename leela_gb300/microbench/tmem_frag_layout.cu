// Layout check (one CTA of 4 warps, every access in bounds): the register layout of
// tcgen05.ld.16x256b.x1 read at each warp's lane-quarter base, and the
// memory layout written by stmatrix.m8n8.x4.trans.  All waits are on
// tcgen05.wait (no spin loops); TMEM: 32 columns allocated and freed.
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__global__ void probe(uint32_t *out_ld, uint16_t *out_stm) {
    __shared__ uint32_t tmem_base;
    __shared__ __align__(16) uint16_t st[4 * 8 * 8];
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(smem_u32(&tmem_base))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tm = tmem_base;
    // TMEM lane (32 warp + lane), column c holds (lane index << 8) | c
    {
        uint32_t v[16];
        for (int c = 0; c < 16; ++c) v[c] = ((uint32_t)(32 * warp + lane) << 8) | (uint32_t)c;
        asm volatile(
            "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
            "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(tm + ((uint32_t)(32 * warp) << 16)),
            "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),
            "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
            : "memory");
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    {
        uint32_t r0, r1, r2, r3;
        asm volatile("tcgen05.ld.sync.aligned.16x256b.x1.b32 {%0,%1,%2,%3}, [%4];"
                     : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                     : "r"(tm + ((uint32_t)(32 * warp) << 16)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        uint32_t *o = out_ld + (warp * 32 + lane) * 4;
        o[0] = r0;
        o[1] = r1;
        o[2] = r2;
        o[3] = r3;
    }
    if (warp == 0) {
        // thread t supplies, for matrix i, the pair (i << 8 | t << 1 | h), h = 0 low, 1 high
        uint32_t q[4];
        for (int i = 0; i < 4; ++i)
            q[i] = ((uint32_t)((i << 8) | (lane << 1) | 0)) | ((uint32_t)((i << 8) | (lane << 1) | 1) << 16);
        for (int k = lane; k < 4 * 8 * 8; k += 32) st[k] = 0xFFFF;
        __syncwarp();
        // threads 8i..8i+7 give the addresses of memory rows 0..7 of matrix i
        const uint32_t addr = smem_u32(&st[(lane / 8) * 64 + (lane % 8) * 8]);
        asm volatile("stmatrix.sync.aligned.m8n8.x4.trans.shared.b16 [%0], {%1,%2,%3,%4};" ::"r"(addr), "r"(q[0]),
                     "r"(q[1]), "r"(q[2]), "r"(q[3])
                     : "memory");
        __syncwarp();
        for (int k = lane; k < 4 * 8 * 8; k += 32) out_stm[k] = st[k];
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tm) : "memory");
}

int main() {
    uint32_t *d_ld;
    uint16_t *d_stm;
    cudaMalloc(&d_ld, 128 * 4 * 4);
    cudaMalloc(&d_stm, 256 * 2);
    probe<<<1, 128>>>(d_ld, d_stm);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        printf("error %s\n", cudaGetErrorString(e));
        return 1;
    }
    uint32_t ld[512];
    uint16_t stm[256];
    cudaMemcpy(ld, d_ld, sizeof ld, cudaMemcpyDeviceToHost);
    cudaMemcpy(stm, d_stm, sizeof stm, cudaMemcpyDeviceToHost);
    // expected (mma accumulator-fragment layout): thread t of warp w gets
    // lane 32w + t/4 columns 2(t%4), 2(t%4)+1, then lane 32w + 8 + t/4, same columns
    int bad_ld = 0;
    for (int w = 0; w < 4; ++w)
        for (int t = 0; t < 32; ++t)
            for (int k = 0; k < 4; ++k) {
                const uint32_t lanei = 32 * w + t / 4 + (k >= 2 ? 8 : 0), col = 2 * (t % 4) + (k & 1);
                const uint32_t want = (lanei << 8) | col, got = ld[(w * 32 + t) * 4 + k];
                if (got != want && bad_ld++ < 8)
                    printf("ld w%d t%d r%d: got lane %u col %u, expected lane %u col %u\n", w, t, k, got >> 8,
                           got & 255, lanei, col);
            }
    // expected: memory row k of matrix i, element j = the value thread
    // t = 4j + k/2 gave as half h = k%2
    int bad_st = 0;
    for (int i = 0; i < 4; ++i)
        for (int k = 0; k < 8; ++k)
            for (int j = 0; j < 8; ++j) {
                const int t = 4 * j + k / 2, h = k % 2;
                const uint16_t want = (uint16_t)((i << 8) | (t << 1) | h), got = stm[i * 64 + k * 8 + j];
                if (got != want && bad_st++ < 8)
                    printf("stm m%d row %d el %d: got %04x expected %04x\n", i, k, j, got, want);
            }
    printf("tcgen05.ld.16x256b layout %s (%d mismatches); stmatrix.trans layout %s (%d mismatches)\n",
           bad_ld ? "DIFFERS" : "as expected", bad_ld, bad_st ? "DIFFERS" : "as expected", bad_st);
    printf("first thread words: %08x %08x %08x %08x\n", ld[0], ld[1], ld[2], ld[3]);
    return 0;
}
