// op_rates.cu -- throughput of the integer instructions the DP kernels are built from, measured
// on the device (bwacuda_measure_op_rate).  Each thread runs 8 independent chains of one
// operation, so the issuing pipe, not the chain latency, sets the rate; an operation that is one
// ALU-pipe instruction runs at the ALU peak (bwacuda_measure_alu_peak), one that takes two runs
// at half of it, and one issued to the FMA pipe (IMAD) at that pipe's rate.  The rates, with the
// instruction counts an ncu pass gives for the same launches (`bench.py --case op-rates`), are
// the basis of the one-instruction-per-operation cell counts the rooflines use.
#include <cuda_runtime.h>

#include "common.cuh"
#include "runtime.h"

namespace bwacuda {
namespace {

constexpr int CHAINS = 8;
constexpr int UNROLL = 16;

// One operation of chain value a; nb is the neighbouring chain's value.  The two idempotent forms
// (a max of two, an and-or) take nb as an operand so that no two steps of a chain fold into one.
template <int OP>
__device__ __forceinline__ uint32_t op(uint32_t a, uint32_t nb, uint32_t b, uint32_t c)
{
    if constexpr (OP == BWACUDA_OPR_VIADDMAX_S32) return (uint32_t)__viaddmax_s32((int)a, (int)b, (int)c);
    if constexpr (OP == BWACUDA_OPR_VIADDMAX_S32_RELU) return (uint32_t)__viaddmax_s32_relu((int)a, (int)b, (int)c);
    if constexpr (OP == BWACUDA_OPR_VIADDMAX_S16X2) return __viaddmax_s16x2(a, b, c);
    if constexpr (OP == BWACUDA_OPR_VIADDMAX_S16X2_RELU) return __viaddmax_s16x2_relu(a, b, c);
    if constexpr (OP == BWACUDA_OPR_VIADDMIN_S16X2) return __viaddmin_s16x2(a, b, c);
    if constexpr (OP == BWACUDA_OPR_VIMAX3_S16X2) return __vimax3_s16x2(a, b, c);
    if constexpr (OP == BWACUDA_OPR_VIMAX3_U16X2) return __vimax3_u16x2(a, b, c);
    if constexpr (OP == BWACUDA_OPR_VIMAX_S16X2_RELU) return __vimax_s16x2_relu(a, nb);
    if constexpr (OP == BWACUDA_OPR_VIMAX3_S32) return (uint32_t)__vimax3_s32((int)a, (int)b, (int)c);
    if constexpr (OP == BWACUDA_OPR_PRMT) return prmt(a, b, c);
    if constexpr (OP == BWACUDA_OPR_C_ADD_MAX) {
        const int x = (int)a + (int)b;
        return (uint32_t)(x > (int)c ? x : (int)c);
    }
    if constexpr (OP == BWACUDA_OPR_IMAD) return a * b + c;
    if constexpr (OP == BWACUDA_OPR_LOP3) return (a & b) | nb;
    (void)nb;
    return a;
}

template <int OP>
__global__ void __launch_bounds__(256) op_rate_kernel(int iters, uint32_t b, uint32_t c, uint32_t *out)
{
    uint32_t a[CHAINS];
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) a[k] = threadIdx.x * (uint32_t)(k + 1) + b;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) {
#pragma unroll
            for (int k = 0; k < CHAINS; ++k) a[k] = op<OP>(a[k], a[(k + 1) % CHAINS], b, c);
        }
    }
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s ^= a[k];
    if (s == 0x9e3779b9u) out[0] = s;  // keeps the chains live
}

template <int OP>
cudaError_t launch(int blocks, int iters, uint32_t *out, cudaStream_t s)
{
    // operands chosen so no chain settles on a constant: b, c mix values across the lanes
    const uint32_t b = OP == BWACUDA_OPR_PRMT ? 0x5140u : (OP == BWACUDA_OPR_IMAD ? 3u : 0x00030005u);
    const uint32_t c = OP == BWACUDA_OPR_PRMT ? 0x3715u : 0x80018001u;
    op_rate_kernel<OP><<<blocks, 256, 0, s>>>(iters, b, c, out);
    return cudaGetLastError();
}

cudaError_t launch_op(int opc, int blocks, int iters, uint32_t *out, cudaStream_t s)
{
    switch (opc) {
    case BWACUDA_OPR_VIADDMAX_S32: return launch<BWACUDA_OPR_VIADDMAX_S32>(blocks, iters, out, s);
    case BWACUDA_OPR_VIADDMAX_S32_RELU: return launch<BWACUDA_OPR_VIADDMAX_S32_RELU>(blocks, iters, out, s);
    case BWACUDA_OPR_VIADDMAX_S16X2: return launch<BWACUDA_OPR_VIADDMAX_S16X2>(blocks, iters, out, s);
    case BWACUDA_OPR_VIADDMAX_S16X2_RELU: return launch<BWACUDA_OPR_VIADDMAX_S16X2_RELU>(blocks, iters, out, s);
    case BWACUDA_OPR_VIADDMIN_S16X2: return launch<BWACUDA_OPR_VIADDMIN_S16X2>(blocks, iters, out, s);
    case BWACUDA_OPR_VIMAX3_S16X2: return launch<BWACUDA_OPR_VIMAX3_S16X2>(blocks, iters, out, s);
    case BWACUDA_OPR_VIMAX3_U16X2: return launch<BWACUDA_OPR_VIMAX3_U16X2>(blocks, iters, out, s);
    case BWACUDA_OPR_VIMAX_S16X2_RELU: return launch<BWACUDA_OPR_VIMAX_S16X2_RELU>(blocks, iters, out, s);
    case BWACUDA_OPR_VIMAX3_S32: return launch<BWACUDA_OPR_VIMAX3_S32>(blocks, iters, out, s);
    case BWACUDA_OPR_PRMT: return launch<BWACUDA_OPR_PRMT>(blocks, iters, out, s);
    case BWACUDA_OPR_C_ADD_MAX: return launch<BWACUDA_OPR_C_ADD_MAX>(blocks, iters, out, s);
    case BWACUDA_OPR_IMAD: return launch<BWACUDA_OPR_IMAD>(blocks, iters, out, s);
    case BWACUDA_OPR_LOP3: return launch<BWACUDA_OPR_LOP3>(blocks, iters, out, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace
}  // namespace bwacuda

using namespace bwacuda;

extern "C" int bwacuda_measure_op_rate(bwacuda_ctx *c, int opc, double *gops)
{
    if (!c || !gops || opc < 0 || opc >= BWACUDA_OPR_COUNT) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    int nsm = 0;
    cudaError_t e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    if (e != cudaSuccess) return cuda_status(e);
    const int blocks = nsm * 8, iters = 1024;
    cudaStream_t s = c->stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if ((e = cudaEventCreate(&e0)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaEventCreate(&e1)) != cudaSuccess) { cudaEventDestroy(e0); return cuda_status(e); }
    uint32_t *out = static_cast<uint32_t *>(c->d_misc.p) + 64;  // scratch word of the context's misc buffer
    float best = 0.f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
        e = cudaEventRecord(e0, s);
        if (e == cudaSuccess) e = launch_op(opc, blocks, iters, out, s);
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && rep > 0 && (best == 0.f || ms < best)) best = ms;  // the first launch warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_status(e);
    const double ops = (double)blocks * 256 * iters * UNROLL * CHAINS;
    *gops = best > 0.f ? ops / (best * 1e-3) / 1e9 : 0.0;
    c->stats.kernel_launches += 4;
    return BWACUDA_OK;
}
