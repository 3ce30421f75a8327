// host_link.cu -- measured host<->device bandwidth over the link the host-buffer calls use
// (NVLink-C2C on Grace-Blackwell): the device reading pinned host memory with 16-byte loads (the
// device-gather route's access), the copy engine's host-to-device copy, and the device writing
// pinned host memory (the result stores of the host-buffer calls).  The end-to-end roofline of a
// host-buffer call is its bytes over these rates.
#include <cuda_runtime.h>

#include "runtime.h"

namespace bwacuda {
namespace {

// Streams n 16-byte words: eight independent loads in flight per thread.
__global__ void __launch_bounds__(256) link_read_kernel(const uint4 *__restrict__ p, size_t n, uint32_t *out)
{
    uint32_t acc = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 7 * stride < n; i += 8 * stride) {
        uint4 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = p[i + u * stride];
#pragma unroll
        for (int u = 0; u < 8; ++u) acc ^= v[u].x ^ v[u].y ^ v[u].z ^ v[u].w;
    }
    for (; i < n; i += stride) {
        const uint4 v = p[i];
        acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
    if (acc == 0x9e3779b9u) out[0] = acc;  // keeps the loads live
}

__global__ void __launch_bounds__(256) link_write_kernel(uint4 *__restrict__ p, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        p[i] = make_uint4((uint32_t)i, 0u, 0u, 0u);
}

// Best of three timed runs after one warm-up; ms of one run.
template <class Fn>
cudaError_t best_ms(cudaStream_t s, const Fn &fn, float *ms)
{
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float best = 0.f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
        e = cudaEventRecord(e0, s);
        if (e == cudaSuccess) e = fn();
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float t = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
        if (e == cudaSuccess && rep > 0 && (best == 0.f || t < best)) best = t;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    *ms = best;
    return e;
}

}  // namespace
}  // namespace bwacuda

using namespace bwacuda;

extern "C" int bwacuda_measure_host_link(bwacuda_ctx *c, size_t bytes, double *read_gbs, double *copy_gbs,
                                         double *write_gbs)
{
    if (!c || !read_gbs || !copy_gbs || !write_gbs || bytes < (1u << 20) || bytes > (size_t(16) << 30))
        return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    bytes &= ~size_t(15);
    const size_t n = bytes / 16;
    int nsm = 0;
    cudaError_t e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    if (e != cudaSuccess) return cuda_status(e);
    void *host = nullptr, *dev = nullptr;
    if ((e = cudaMallocHost(&host, bytes)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaMalloc(&dev, bytes)) != cudaSuccess) { cudaFreeHost(host); return cuda_status(e); }
    cudaStream_t s = c->stream;
    uint32_t *out = static_cast<uint32_t *>(c->d_misc.p) + 64;  // scratch word of the context's misc buffer
    const uint32_t grid = (uint32_t)nsm * 4;
    float t_read = 0.f, t_copy = 0.f, t_write = 0.f;
    e = cudaMemsetAsync(dev, 1, bytes, s);
    if (e == cudaSuccess)
        e = best_ms(s, [&]() {
            link_write_kernel<<<grid, 256, 0, s>>>(static_cast<uint4 *>(host), n);
            return cudaGetLastError();
        }, &t_write);
    if (e == cudaSuccess)
        e = best_ms(s, [&]() {
            link_read_kernel<<<grid, 256, 0, s>>>(static_cast<const uint4 *>(host), n, out);
            return cudaGetLastError();
        }, &t_read);
    if (e == cudaSuccess)
        e = best_ms(s, [&]() { return cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, s); }, &t_copy);
    const cudaError_t e2 = cudaStreamSynchronize(s);
    cudaFree(dev);
    cudaFreeHost(host);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return cuda_status(e);
    auto gbs = [&](float ms) { return ms > 0.f ? (double)bytes / (ms * 1e-3) / 1e9 : 0.0; };
    *read_gbs = gbs(t_read);
    *copy_gbs = gbs(t_copy);
    *write_gbs = gbs(t_write);
    c->stats.kernel_launches += 8;
    return BWACUDA_OK;
}
