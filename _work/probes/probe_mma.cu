// probe_mma.cu -- tensor-core throughput of warp-level mma.sync on sm_103a for the
// FP64-emulation design: bf16 m16n8k16 (f32 accumulate) and s8 m16n8k32 (s32
// accumulate). Not part of the library. Register-only operands, bounded loops,
// one in-bounds store per thread.
#include <cstdio>
#include <cuda_runtime.h>

__global__ void mma_bf16(float *out, int iters)
{
    unsigned a0 = 0x3f803f80u ^ threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, b0 = 0x3f803f80u, b1 = b0 + 7;
    float c[4][4] = {};
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int q = 0; q < 4; ++q)
            asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
                         : "+f"(c[q][0]), "+f"(c[q][1]), "+f"(c[q][2]), "+f"(c[q][3])
                         : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }
    float s = 0;
    for (int q = 0; q < 4; ++q) s += c[q][0] + c[q][1] + c[q][2] + c[q][3];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void mma_s8(int *out, int iters)
{
    unsigned a0 = 0x01010101u ^ threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, b0 = 0x01020304u, b1 = b0 + 5;
    int c[4][4] = {};
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int q = 0; q < 4; ++q)
            asm volatile("mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
                         : "+r"(c[q][0]), "+r"(c[q][1]), "+r"(c[q][2]), "+r"(c[q][3])
                         : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }
    int s = 0;
    for (int q = 0; q < 4; ++q) s += c[q][0] + c[q][1] + c[q][2] + c[q][3];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int main()
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    const int blocks = sms * 4, threads = 256, iters = 4096;
    float *of;
    int *oi;
    if (cudaMalloc(&of, sizeof(float) * blocks * threads) != cudaSuccess) return 1;
    if (cudaMalloc(&oi, sizeof(int) * blocks * threads) != cudaSuccess) return 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float ms;
    const double warps = blocks * (threads / 32.0);
    for (int rep = 0; rep < 2; ++rep) {
        mma_bf16<<<blocks, threads>>>(of, iters);
        cudaEventRecord(e0);
        mma_bf16<<<blocks, threads>>>(of, iters);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess) return 2;
        cudaEventElapsedTime(&ms, e0, e1);
        printf("mma.sync bf16 m16n8k16: %.1f TFLOP/s\n", 2.0 * 16 * 8 * 16 * 4.0 * iters * warps / ms / 1e9);
        mma_s8<<<blocks, threads>>>(oi, iters);
        cudaEventRecord(e0);
        mma_s8<<<blocks, threads>>>(oi, iters);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess) return 2;
        cudaEventElapsedTime(&ms, e0, e1);
        printf("mma.sync s8 m16n8k32:   %.1f TOP/s\n", 2.0 * 16 * 8 * 32 * 4.0 * iters * warps / ms / 1e9);
    }
    return 0;
}
