// ctd_probe.cu -- measurement probes for the roofline denominators (bench only).
//
// The residue kernels are bound by the 32-bit integer ALU issue rate, which
// MEASURED_PEAKS-style copy/GEMM peaks do not describe.  This kernel runs
// eight independent dependency chains per thread alternating a 32-bit add
// and a 32-bit xor (one IADD3 and one LOP3 each: an add and an xor cannot be
// fused into one instruction), with runtime operands so nothing folds, and
// reports integer instructions per second.  Not part of the trial-factoring
// path; libctd_probe.so is loaded only by bench.py.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

__global__ void __launch_bounds__(256) int_chains(uint32_t *out, uint32_t iters, uint32_t y, uint32_t z)
{
    uint32_t a0 = threadIdx.x, a1 = a0 ^ 0x9e3779b9u, a2 = a0 + 7u, a3 = a0 * 3u;
    uint32_t a4 = a0 ^ y, a5 = a0 + z, a6 = a0 ^ 0x85ebca6bu, a7 = a0 + 0x27d4eb2fu;
    for (uint32_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            a0 = (a0 + y) ^ z;
            a1 = (a1 + y) ^ z;
            a2 = (a2 + y) ^ z;
            a3 = (a3 + y) ^ z;
            a4 = (a4 + y) ^ z;
            a5 = (a5 + y) ^ z;
            a6 = (a6 + y) ^ z;
            a7 = (a7 + y) ^ z;
        }
    }
    uint32_t s = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
    if (s == 0x12345678u)  // practically never; keeps the chains live
        out[blockIdx.x] = s;
}

// Integer ALU pipe alone: predicate-accumulating compares (ISETP with an OR
// into the destination predicate), which only the ALU pipe executes -- the
// instruction the compare-bound residue walks are made of.  Eight
// independent predicate chains, 128 compares per iteration.
__global__ void __launch_bounds__(256) isetp_chains(uint32_t *out, uint32_t iters, uint32_t y)
{
    uint32_t a = threadIdx.x * 0x9e3779b9u + y, flags = 0;
    for (uint32_t i = 0; i < iters; ++i) {
        uint32_t f;
        asm volatile(
            "{\n\t.reg .pred q<8>;\n\t"
            "setp.eq.u32 q0, %1, %2;\n\tsetp.eq.u32 q1, %1, %3;\n\tsetp.eq.u32 q2, %1, %4;\n\t"
            "setp.eq.u32 q3, %1, %5;\n\tsetp.eq.u32 q4, %1, %6;\n\tsetp.eq.u32 q5, %1, %7;\n\t"
            "setp.eq.u32 q6, %1, %8;\n\tsetp.eq.u32 q7, %1, %9;\n\t"
#define CTD_PROBE_8                                                                                          \
            "setp.eq.or.u32 q0, %1, %9, q0;\n\tsetp.eq.or.u32 q1, %1, %8, q1;\n\t"                        \
            "setp.eq.or.u32 q2, %1, %7, q2;\n\tsetp.eq.or.u32 q3, %1, %6, q3;\n\t"                        \
            "setp.eq.or.u32 q4, %1, %5, q4;\n\tsetp.eq.or.u32 q5, %1, %4, q5;\n\t"                        \
            "setp.eq.or.u32 q6, %1, %3, q6;\n\tsetp.eq.or.u32 q7, %1, %2, q7;\n\t"
            CTD_PROBE_8 CTD_PROBE_8 CTD_PROBE_8 CTD_PROBE_8 CTD_PROBE_8 CTD_PROBE_8 CTD_PROBE_8 CTD_PROBE_8
            CTD_PROBE_8 CTD_PROBE_8 CTD_PROBE_8 CTD_PROBE_8 CTD_PROBE_8 CTD_PROBE_8 CTD_PROBE_8
#undef CTD_PROBE_8
            "or.pred q0, q0, q1;\n\tor.pred q2, q2, q3;\n\tor.pred q4, q4, q5;\n\tor.pred q6, q6, q7;\n\t"
            "or.pred q0, q0, q2;\n\tor.pred q4, q4, q6;\n\tor.pred q0, q0, q4;\n\t"
            "selp.u32 %0, 1, 0, q0;\n\t}"
            : "=r"(f)
            : "r"(a), "r"(y), "r"(y + 1), "r"(y + 2), "r"(y + 3), "r"(y + 4), "r"(y + 5), "r"(y + 6), "r"(y + 7));
        flags |= f;
        a += 0x61c88647u;
    }
    if (flags == 0x12345678u)  // never: keeps the compares live
        out[blockIdx.x] = flags;
}

// Integer multiply pipe: eight independent chains of 32-bit multiply-adds
// (IMAD, a = a * y + z), the instruction the Smarandache steps are built
// from; 128 multiply-adds per iteration.
__global__ void __launch_bounds__(256) imad_chains(uint32_t *out, uint32_t iters, uint32_t y, uint32_t z)
{
    uint32_t a0 = threadIdx.x, a1 = a0 ^ 0x9e3779b9u, a2 = a0 + 7u, a3 = a0 * 3u;
    uint32_t a4 = a0 ^ y, a5 = a0 + z, a6 = a0 ^ 0x85ebca6bu, a7 = a0 + 0x27d4eb2fu;
    for (uint32_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            a0 = a0 * y + z;
            a1 = a1 * y + z;
            a2 = a2 * y + z;
            a3 = a3 * y + z;
            a4 = a4 * y + z;
            a5 = a5 * y + z;
            a6 = a6 * y + z;
            a7 = a7 * y + z;
        }
    }
    uint32_t s = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
    if (s == 0x12345678u)  // practically never; keeps the chains live
        out[blockIdx.x] = s;
}

}  // namespace

extern "C" {

// 32-bit integer multiply-adds per second over a ~0.5 s run on `device`
// (8 chains x 16 unrolled x iters per thread).  Returns 0 on success.
int ctd_probe_imad_peak(int device, double *imad_per_s, double *seconds)
{
    if (cudaSetDevice(device) != cudaSuccess)
        return -2;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    uint32_t *out = nullptr;
    const int block = 256, grid = sms * 8;
    if (cudaMalloc(&out, grid * sizeof(uint32_t)) != cudaSuccess)
        return -3;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const uint32_t iters = 2048;
    imad_chains<<<grid, block>>>(out, 64, 0x1234567u, 0x89abcdefu);  // warm-up
    cudaEventRecord(e0);
    const int reps = 8;
    for (int r = 0; r < reps; ++r)
        imad_chains<<<grid, block>>>(out, iters, 0x1234567u + 2 * r, 0x89abcdefu);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f)
        return -2;
    const double instr = 8.0 * 16 * (double)iters * block * grid * reps;
    *imad_per_s = instr / (ms * 1e-3);
    if (seconds)
        *seconds = ms * 1e-3;
    return 0;
}

// Predicate compares per second (ALU pipe) over a ~0.5 s run on `device`
// (128 compares per iteration; the dozen or/select/add/loop instructions
// around them are not counted, so this understates the pipe by a few
// percent).  Returns 0 on success.
int ctd_probe_alu_peak(int device, double *compares_per_s, double *seconds)
{
    if (cudaSetDevice(device) != cudaSuccess)
        return -2;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    uint32_t *out = nullptr;
    const int block = 256, grid = sms * 8;
    if (cudaMalloc(&out, grid * sizeof(uint32_t)) != cudaSuccess)
        return -3;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const uint32_t iters = 1 << 12;
    isetp_chains<<<grid, block>>>(out, 64, 0x1234567u);  // warm-up
    cudaEventRecord(e0);
    const int reps = 8;
    for (int r = 0; r < reps; ++r)
        isetp_chains<<<grid, block>>>(out, iters, 0x1234567u + 16 * r);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f)
        return -2;
    const double instr = 128.0 * (double)iters * block * grid * reps;
    *compares_per_s = instr / (ms * 1e-3);
    if (seconds)
        *seconds = ms * 1e-3;
    return 0;
}

// Integer ALU instructions per second over a ~0.5 s run on `device`
// (2 instructions x 8 chains x 16 unrolled x iters per thread).  Returns 0
// on success.
int ctd_probe_int_peak(int device, double *int_ops_per_s, double *seconds)
{
    if (cudaSetDevice(device) != cudaSuccess)
        return -2;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    uint32_t *out = nullptr;
    const int block = 256, grid = sms * 8;
    if (cudaMalloc(&out, grid * sizeof(uint32_t)) != cudaSuccess)
        return -3;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const uint32_t iters = 4096;
    int_chains<<<grid, block>>>(out, 64, 0x1234567u, 0x89abcdefu);  // warm-up
    cudaEventRecord(e0);
    const int reps = 8;
    for (int r = 0; r < reps; ++r)
        int_chains<<<grid, block>>>(out, iters, 0x1234567u + r, 0x89abcdefu);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f)
        return -2;
    const double instr = 2.0 * 8 * 16 * (double)iters * block * grid * reps;
    *int_ops_per_s = instr / (ms * 1e-3);
    if (seconds)
        *seconds = ms * 1e-3;
    return 0;
}

}  // extern "C"
