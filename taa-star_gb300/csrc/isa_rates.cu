// isa_rates.cu - a stand-alone measurement (not part of the library): the
// issue rate of packed FP32 (fma.rn.f32x2), packed FP16 (fma.rn.f16x2) and
// scalar FP32 (fma.rn.f32) FMAs on this GPU, in warp instructions and in FMA
// lanes per cycle per SM.  Every thread keeps eight independent chains in
// registers; nothing touches memory but one store the compiler cannot drop.
// It backs the choice of packed FP32 over packed FP16 for the fast resolve:
// where both packed forms issue at the same rate, FP16 arithmetic buys no
// throughput.  Built and run by `python bench.py --isa-rates`; prints one JSON
// line.
#include <cuda_fp16.h>

#include <cstdint>
#include <cstdio>

namespace {
constexpr int kIters = 4096, kChains = 8;

__global__ void fma_f32x2(float* out, float s) {
    unsigned long long a[kChains], m, c;
    for (int i = 0; i < kChains; ++i) {
        const float x = s + (float)threadIdx.x + (float)i;
        asm("mov.b64 %0, {%1, %2};" : "=l"(a[i]) : "f"(x), "f"(x + 1.f));
    }
    asm("mov.b64 %0, {%1, %2};" : "=l"(m) : "f"(0.999f), "f"(0.999f));
    asm("mov.b64 %0, {%1, %2};" : "=l"(c) : "f"(0.001f), "f"(0.001f));
    for (int it = 0; it < kIters; ++it) {
#pragma unroll
        for (int i = 0; i < kChains; ++i) asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(a[i]) : "l"(m), "l"(c));
    }
    float r = 0.f;
    for (int i = 0; i < kChains; ++i) {
        float lo, hi;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a[i]));
        r += lo + hi;
    }
    if (r == 12345.f) out[0] = r;
}

__global__ void fma_f16x2(float* out, float s) {
    uint32_t a[kChains];
    for (int i = 0; i < kChains; ++i) {
        const __half2 h = __floats2half2_rn(s + (float)i, s + (float)i + 1.f);
        a[i] = *reinterpret_cast<const uint32_t*>(&h);
    }
    const __half2 mh = __floats2half2_rn(0.999f, 0.999f), ch = __floats2half2_rn(0.001f, 0.001f);
    const uint32_t m = *reinterpret_cast<const uint32_t*>(&mh), c = *reinterpret_cast<const uint32_t*>(&ch);
    for (int it = 0; it < kIters; ++it) {
#pragma unroll
        for (int i = 0; i < kChains; ++i) asm volatile("fma.rn.f16x2 %0, %0, %1, %2;" : "+r"(a[i]) : "r"(m), "r"(c));
    }
    float r = 0.f;
    for (int i = 0; i < kChains; ++i) {
        const __half2 h = *reinterpret_cast<const __half2*>(&a[i]);
        r += __low2float(h) + __high2float(h);
    }
    if (r == 12345.f) out[0] = r;
}

__global__ void fma_f32(float* out, float s) {
    float a[kChains];
    for (int i = 0; i < kChains; ++i) a[i] = s + (float)threadIdx.x + (float)i;
    for (int it = 0; it < kIters; ++it) {
#pragma unroll
        for (int i = 0; i < kChains; ++i) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(a[i]) : "f"(0.999f), "f"(0.001f));
    }
    float r = 0.f;
    for (int i = 0; i < kChains; ++i) r += a[i];
    if (r == 12345.f) out[0] = r;
}
}  // namespace

int main() {
    int sms = 0, khz = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, 0);
    float* out = nullptr;
    if (cudaMalloc(&out, sizeof(float)) != cudaSuccess) return 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256;
    const char* names[3] = {"fma.rn.f32x2", "fma.rn.f16x2", "fma.rn.f32"};
    const int lanes[3] = {64, 64, 32};  // FMAs per warp instruction
    printf("{\"sms\": %d, \"max_clock_mhz\": %d", sms, khz / 1000);
    for (int k = 0; k < 3; ++k) {
        float ms = 0.f;
        for (int rep = 0; rep < 3; ++rep) {  // the last of three launches
            cudaEventRecord(e0);
            if (k == 0) fma_f32x2<<<blocks, threads>>>(out, 1.f);
            else if (k == 1) fma_f16x2<<<blocks, threads>>>(out, 1.f);
            else fma_f32<<<blocks, threads>>>(out, 1.f);
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&ms, e0, e1);
        }
        if (cudaGetLastError() != cudaSuccess) return 1;
        const double warp_inst = (double)blocks * threads / 32 * kIters * kChains;
        const double per_cycle = warp_inst / sms / (ms * 1e-3 * khz * 1e3);
        printf(", \"%s\": {\"warp_inst_per_cycle_per_sm\": %.3f, \"fma_lanes_per_cycle_per_sm\": %.1f, \"ms\": %.3f}",
               names[k], per_cycle, per_cycle * lanes[k], ms);
    }
    printf(", \"clock\": \"cycles counted at the maximum SM clock\"}\n");
    cudaFree(out);
    return 0;
}
