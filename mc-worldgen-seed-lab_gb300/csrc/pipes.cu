/* pipes.cu -- throughput microbenchmarks of the GPU pipes the biome path uses.
 *
 * The roofline of this path is not HBM or tensor cores: it is FP64 (26.1/26.2 lattice math, every
 * version's coordinate math), FP32 (26.3 lattice math) and integer (RNG, R-tree) issue.  The host's
 * measured-peaks file carries only HBM and bf16 GEMM, so these kernels measure the missing pipe peaks on
 * the same device, the way the reference calibrates its FFMA rate
 * (crack/src/gpu_biomes/bench_gpu_biomes.cu:26-52).  Each thread runs 8 independent dependency chains so
 * the pipe, not latency, bounds the loop; inline PTX keeps each operation from being folded away.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "launch.h"

namespace mg {

#define CHAINS 8

template <int OP>
__global__ void __launch_bounds__(256) k_pipe(int iters, unsigned long long *sink) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    float f[CHAINS];
    double d[CHAINS];
    uint32_t u[CHAINS];
    uint64_t w[CHAINS];
    int acc = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; c++) {
        f[c] = 1.0f + (float)(t + c) * 1e-7f;
        d[c] = 1.0 + (double)(t + c) * 1e-9 + 0.25 * c;
        u[c] = (uint32_t)(t * 2654435761u + c);
        w[c] = (uint64_t)t * 0x9E3779B97F4A7C15ULL + (uint64_t)c;
    }
    const float fb = 0.9999999f, fc = 1e-7f;
    const double db = 0.9999999999, dc = 1e-12;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < CHAINS; c++) {
            if (OP == 0) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(f[c]) : "f"(fb), "f"(fc));
            if (OP == 1) asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(d[c]) : "d"(db), "d"(dc));
            if (OP == 2) asm volatile("add.rn.f64 %0, %0, %1;" : "+d"(d[c]) : "d"(dc));
            if (OP == 3) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(u[c]) : "r"(0xDEECE66Du), "r"(11u));
            /* conversions: each result feeds the next conversion of its chain through one integer op on
             * its bits, so no conversion is loop-invariant or dead */
            if (OP == 4) {
                int r;
                asm volatile("cvt.rmi.s32.f64 %0, %1;" : "=r"(r) : "d"(d[c]));
                d[c] = __hiloint2double(__double2hiint(d[c]), __double2loint(d[c]) ^ r);
            }
            if (OP == 5) {
                const int x = __double2loint(d[c]) + 1;
                asm volatile("cvt.rn.f64.s32 %0, %1;" : "=d"(d[c]) : "r"(x));
            }
            if (OP == 6) {
                float r;
                asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(r) : "d"(d[c]));
                d[c] = __hiloint2double(__double2hiint(d[c]), __double2loint(d[c]) ^ __float_as_int(r));
            }
            if (OP == 7) asm volatile("mad.lo.u64 %0, %0, %1, %2;" : "+l"(w[c]) : "l"(0x5DEECE66DULL), "l"(11ULL));
            if (OP == 8) {
                double r;
                asm volatile("cvt.rn.f64.s64 %0, %1;" : "=d"(r) : "l"(w[c]));
                w[c] = (uint64_t)__double_as_longlong(r) ^ 0x5DEEu;
            }
            if (OP == 9) {
                double r;
                asm volatile("cvt.f64.f32 %0, %1;" : "=d"(r) : "f"(f[c]));
                f[c] = __int_as_float(__double2hiint(r) ^ 0x5DEE);
            }
        }
    }
    unsigned long long h = (unsigned long long)acc;
#pragma unroll
    for (int c = 0; c < CHAINS; c++)
        h ^= (unsigned long long)__float_as_uint(f[c]) ^ (unsigned long long)__double_as_longlong(d[c]) ^ u[c] ^ w[c];
    if (h == 0x1234567ULL) sink[t] = h; /* never true in practice; keeps the chains live */
}

template <int OP>
static int run_pipe(double *gops) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int nt = 256, nb = sms * 8;
    unsigned long long *sink = nullptr;
    cudaError_t e = cudaMalloc(&sink, sizeof(unsigned long long) * (size_t)nt * nb);
    if (e) return (int)e;
    /* FP64-class operations may be ~64x slower per SM than FP32: size each loop for tens of ms */
    const bool slow = OP != 0 && OP != 3;
    const int iters = slow ? 8192 : 8192 * 4;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_pipe<OP><<<nb, nt>>>(iters / 8, sink); /* warm-up */
    cudaEventRecord(a);
    k_pipe<OP><<<nb, nt>>>(iters, sink);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink);
    if (e) return (int)e;
    const double ops = (double)nt * nb * iters * CHAINS;
    *gops = ops / (ms * 1e-3) / 1e9;
    return (int)cudaGetLastError();
}

int pipe_rate(int pipe, double *gops) {
    switch (pipe) {
    case 0: return run_pipe<0>(gops);
    case 1: return run_pipe<1>(gops);
    case 2: return run_pipe<2>(gops);
    case 3: return run_pipe<3>(gops);
    case 4: return run_pipe<4>(gops);
    case 5: return run_pipe<5>(gops);
    case 6: return run_pipe<6>(gops);
    case 7: return run_pipe<7>(gops);
    case 8: return run_pipe<8>(gops);
    case 9: return run_pipe<9>(gops);
    default: return (int)cudaErrorInvalidValue;
    }
}

}  // namespace mg
