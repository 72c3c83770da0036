// FMA throughput probe (FP64 and FP32): eight independent FMA chains per thread, all in
// registers, over 8 CTAs of 256 threads per SM.  A diagnostic for the roofline argument:
// it is not part of libgDMR.
#include <cstdio>
template <class T> __global__ void k(T *out, T a, T b, int iters) {
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
template <class T> void run(const char *name, int iters) {
    int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    int blocks = sms * 8, threads = 256;
    T *out; cudaMalloc(&out, sizeof(T) * blocks * threads);
    k<T><<<blocks, threads>>>(out, (T)0.999, (T)0.001, 10);
    cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
    cudaEventRecord(a);
    k<T><<<blocks, threads>>>(out, (T)0.999, (T)0.001, iters);
    cudaEventRecord(b); cudaEventSynchronize(b);
    float ms; cudaEventElapsedTime(&ms, a, b);
    double flops = 2.0 * 8 * iters * (double)blocks * threads;
    printf("%s: %.3f TFLOP/s (%d SMs, %.2f ms)\n", name, flops / ms / 1e9, sms, ms);
    cudaFree(out);
}
int main() { run<double>("fp64 fma", 2000); run<float>("fp32 fma", 20000); return 0; }
