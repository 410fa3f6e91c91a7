// Host side of the learned inverse-CDF sampler network: parameter storage,
// batched inference on host arrays, one-batch gradients (for checks against
// the CPU restatement) and the Adam training loop over a device-resident
// dataset.  All compute is in the kernels of mlp.cu.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "mlp.cuh"
#include "../../include/particulator_gb300.h"

namespace pcl {
namespace mlp {

static_assert(kNParam == PCL_MLP_NPARAM, "header constant out of date");

struct Handle {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    float* P = nullptr; float* G = nullptr; float* M = nullptr; float* V = nullptr;
    __nv_bfloat16* W2 = nullptr; __nv_bfloat16* W3 = nullptr;
    // batch buffers
    long long cap = 0;
    float* X = nullptr; float* T = nullptr; float* Y = nullptr;
    TrainBuf tb{};
    // dataset
    float* Xall = nullptr; float* Tall = nullptr;
    long long nall = 0, nall_cap = 0;
    double* d_loss = nullptr;
    int* d_err = nullptr;
    long long adam_t = 0;
    std::string err;
};

#define MCK(call)                                                                  \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            h->err = std::string(#call) + ": " + cudaGetErrorString(e_);            \
            return PCL_ERR_CUDA;                                                   \
        }                                                                          \
    } while (0)

static void free_batch(Handle* h) {
    cudaFree(h->X); cudaFree(h->T); cudaFree(h->Y);
    cudaFree(h->tb.z1); cudaFree(h->tb.z2); cudaFree(h->tb.z3);
    cudaFree(h->tb.h1); cudaFree(h->tb.h2); cudaFree(h->tb.dz2); cudaFree(h->tb.dz3);
    h->X = h->T = h->Y = nullptr;
    h->tb = TrainBuf{};
    h->cap = 0;
}

static int ensure_batch(Handle* h, long long n) {
    if (n <= h->cap) return PCL_OK;
    MCK(cudaStreamSynchronize(h->stream));
    free_batch(h);
    long long c = std::max<long long>(n, 1024);
    MCK(cudaMalloc(&h->X, sizeof(float) * 2 * c));
    MCK(cudaMalloc(&h->T, sizeof(float) * c));
    MCK(cudaMalloc(&h->Y, sizeof(float) * c));
    MCK(cudaMalloc(&h->tb.z1, sizeof(float) * kH * c));
    MCK(cudaMalloc(&h->tb.z2, sizeof(float) * kH * c));
    MCK(cudaMalloc(&h->tb.z3, sizeof(float) * kH * c));
    MCK(cudaMalloc(&h->tb.h1, sizeof(__nv_bfloat16) * kH * c));
    MCK(cudaMalloc(&h->tb.h2, sizeof(__nv_bfloat16) * kH * c));
    MCK(cudaMalloc(&h->tb.dz2, sizeof(__nv_bfloat16) * kH * c));
    MCK(cudaMalloc(&h->tb.dz3, sizeof(__nv_bfloat16) * kH * c));
    h->cap = c;
    return PCL_OK;
}

static int set_attrs(Handle* h) {
    MCK(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kFwdSmem)));
    MCK(cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kInferSmem)));
    MCK(cudaFuncSetAttribute(k_mlp_bwd_a, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kBwdASmem)));
    MCK(cudaFuncSetAttribute(k_mlp_bwd_w, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kBwdWSmem)));
    return PCL_OK;
}

Net net_of(const Handle* h) { return Net{h->P, h->W2, h->W3}; }

// training forward launch (targets T)
static int forward(Handle* h, const float* X, long long n, float* Y, const float* T) {
    long long ntiles = (n + kH - 1) / kH;
    int grid = int(std::min<long long>(ntiles, 2ll * h->sm_count));
    if (grid < 1) return PCL_OK;
    k_mlp_forward<<<grid, 128, kFwdSmem, h->stream>>>(net_of(h), X, n, Y, h->tb, T, h->G, h->d_loss, h->d_err);
    MCK(cudaGetLastError());
    return PCL_OK;
}

// forward + backward of one batch already in h->X / h->T; gradients in h->G
static int grad_batch(Handle* h, long long n) {
    MCK(cudaMemsetAsync(h->G, 0, sizeof(float) * kNParam, h->stream));
    int rc = forward(h, h->X, n, nullptr, h->T);
    if (rc) return rc;
    long long ntiles = (n + kH - 1) / kH;
    int grid = int(std::min<long long>(ntiles, 2ll * h->sm_count));
    k_mlp_bwd_a<<<grid, 128, kBwdASmem, h->stream>>>(net_of(h), h->X, n, h->tb, h->G, h->d_err);
    MCK(cudaGetLastError());
    int gw = int(std::min<long long>(ntiles, (long long)h->sm_count));
    k_mlp_bwd_w<<<gw, 128, kBwdWSmem, h->stream>>>(n, h->tb, h->G, h->d_err);
    MCK(cudaGetLastError());
    return PCL_OK;
}

static int check_err(Handle* h) {
    int e = 0;
    MCK(cudaMemcpyAsync(&e, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MCK(cudaStreamSynchronize(h->stream));
    if (e) {
        h->err = "tensor-core wait timed out";
        return PCL_ERR_TIMEOUT;
    }
    return PCL_OK;
}

static uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Several networks on the same rows, min(cap, *n_dev) of them, the count read
// on the device (no host read-back, so the launch can sit in a captured
// graph): network k writes Y + k * ystride.  One launch per kMaxNets
// networks, a grid of at most one block per SM per network walking the tiles.
cudaError_t infer_multi(void* const* handles, int nnets, const float* X, const unsigned long long* n_dev,
                        long long cap, float* Y, long long ystride, cudaStream_t stream) {
    if (cap <= 0 || nnets <= 0) return cudaSuccess;
    const Handle* h0 = static_cast<const Handle*>(handles[0]);
    long long ntiles = (cap + kH - 1) / kH;
    int gx = int(std::min<long long>(ntiles, (long long)h0->sm_count));
    for (int k0 = 0; k0 < nnets; k0 += kMaxNets) {
        NetSet ns{};
        const int m = std::min(kMaxNets, nnets - k0);
        for (int i = 0; i < m; ++i) {
            ns.net[i] = net_of(static_cast<const Handle*>(handles[k0 + i]));
            ns.Y[i] = Y + (long long)(k0 + i) * ystride;
        }
        k_mlp_infer<<<dim3(gx, m), kInferThreads, kInferSmem, stream>>>(ns, X, cap, n_dev, h0->d_err);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace mlp
}  // namespace pcl

using namespace pcl::mlp;

extern "C" {

int pcl_mlp_create(int device, uint64_t seed, void** out) {
    if (!out) return PCL_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PCL_ERR_CUDA;
    if (device < 0 || device >= ndev) return PCL_ERR_INVALID;
    Handle* h = new Handle();
    h->device = device;
    if (cudaSetDevice(device) != cudaSuccess) { delete h; return PCL_ERR_CUDA; }
    cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&h->P, sizeof(float) * kNParam) != cudaSuccess ||
        cudaMalloc(&h->G, sizeof(float) * kNParam) != cudaSuccess ||
        cudaMalloc(&h->M, sizeof(float) * kNParam) != cudaSuccess ||
        cudaMalloc(&h->V, sizeof(float) * kNParam) != cudaSuccess ||
        cudaMalloc(&h->W2, sizeof(__nv_bfloat16) * kH * kH) != cudaSuccess ||
        cudaMalloc(&h->W3, sizeof(__nv_bfloat16) * kH * kH) != cudaSuccess ||
        cudaMalloc(&h->d_loss, sizeof(double)) != cudaSuccess ||
        cudaMalloc(&h->d_err, sizeof(int)) != cudaSuccess || set_attrs(h) != PCL_OK) {
        pcl_mlp_destroy(h);
        return PCL_ERR_CUDA;
    }
    // He-uniform initialisation from a seeded 64-bit generator; biases zero
    std::vector<float> p(kNParam, 0.0f);
    uint64_t s = seed ^ 0x5EED5EED5EEDull;
    auto uni = [&](float a) { return a * float(2.0 * (double(splitmix(s) >> 11) * 0x1.0p-53) - 1.0); };
    for (int i = 0; i < 2 * kH; ++i) p[oW1 + i] = uni(std::sqrt(6.0f / 2.0f));
    for (int i = 0; i < kH * kH; ++i) p[oW2 + i] = uni(std::sqrt(6.0f / kH));
    for (int i = 0; i < kH * kH; ++i) p[oW3 + i] = uni(std::sqrt(6.0f / kH));
    for (int i = 0; i < kH; ++i) p[ow4 + i] = uni(std::sqrt(3.0f / kH));
    int rc = pcl_mlp_set_params(h, p.data(), kNParam);
    if (rc) { pcl_mlp_destroy(h); return rc; }
    *out = h;
    return PCL_OK;
}

void pcl_mlp_destroy(void* mh) {
    if (!mh) return;
    Handle* h = static_cast<Handle*>(mh);
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_batch(h);
    cudaFree(h->P); cudaFree(h->G); cudaFree(h->M); cudaFree(h->V); cudaFree(h->W2); cudaFree(h->W3);
    cudaFree(h->Xall); cudaFree(h->Tall); cudaFree(h->d_loss); cudaFree(h->d_err);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

const char* pcl_mlp_last_error(void* mh) {
    if (!mh) return "null network handle";
    return static_cast<Handle*>(mh)->err.c_str();
}

int pcl_mlp_set_params(void* mh, const float* params, int64_t n) {
    Handle* h = static_cast<Handle*>(mh);
    if (!h || !params || n != kNParam) return PCL_ERR_INVALID;
    MCK(cudaSetDevice(h->device));
    MCK(cudaMemcpyAsync(h->P, params, sizeof(float) * kNParam, cudaMemcpyHostToDevice, h->stream));
    MCK(cudaMemsetAsync(h->M, 0, sizeof(float) * kNParam, h->stream));
    MCK(cudaMemsetAsync(h->V, 0, sizeof(float) * kNParam, h->stream));
    MCK(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
    k_mlp_sync_bf16<<<64, 256, 0, h->stream>>>(h->P, h->W2, h->W3);
    MCK(cudaGetLastError());
    MCK(cudaStreamSynchronize(h->stream));
    h->adam_t = 0;
    return PCL_OK;
}

int pcl_mlp_get_params(void* mh, float* params, int64_t n) {
    Handle* h = static_cast<Handle*>(mh);
    if (!h || !params || n != kNParam) return PCL_ERR_INVALID;
    MCK(cudaSetDevice(h->device));
    MCK(cudaMemcpyAsync(params, h->P, sizeof(float) * kNParam, cudaMemcpyDeviceToHost, h->stream));
    MCK(cudaStreamSynchronize(h->stream));
    return PCL_OK;
}

int pcl_mlp_forward(void* mh, int64_t n, const float* x, float* y) {
    Handle* h = static_cast<Handle*>(mh);
    if (!h || n < 0 || (n > 0 && (!x || !y))) return PCL_ERR_INVALID;
    if (n == 0) return PCL_OK;
    MCK(cudaSetDevice(h->device));
    int rc = ensure_batch(h, n);
    if (rc) return rc;
    MCK(cudaMemcpyAsync(h->X, x, sizeof(float) * 2 * n, cudaMemcpyHostToDevice, h->stream));
    void* one[1] = {h};   // the inference kernel of the step's learned round
    MCK(infer_multi(one, 1, h->X, nullptr, n, h->Y, n, h->stream));
    MCK(cudaMemcpyAsync(y, h->Y, sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream));
    return check_err(h);
}

int pcl_mlp_gradient(void* mh, int64_t n, const float* x, const float* t, float* grad, double* loss) {
    Handle* h = static_cast<Handle*>(mh);
    if (!h || n <= 0 || !x || !t || !grad) return PCL_ERR_INVALID;
    MCK(cudaSetDevice(h->device));
    int rc = ensure_batch(h, n);
    if (rc) return rc;
    MCK(cudaMemcpyAsync(h->X, x, sizeof(float) * 2 * n, cudaMemcpyHostToDevice, h->stream));
    MCK(cudaMemcpyAsync(h->T, t, sizeof(float) * n, cudaMemcpyHostToDevice, h->stream));
    MCK(cudaMemsetAsync(h->d_loss, 0, sizeof(double), h->stream));
    if ((rc = grad_batch(h, n))) return rc;
    MCK(cudaMemcpyAsync(grad, h->G, sizeof(float) * kNParam, cudaMemcpyDeviceToHost, h->stream));
    double l = 0.0;
    MCK(cudaMemcpyAsync(&l, h->d_loss, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    rc = check_err(h);
    if (loss) *loss = l;
    return rc;
}

int pcl_mlp_train(void* mh, int64_t n, const float* x, const float* t, int64_t steps, int32_t batch, double lr,
                  uint64_t seed, double* loss) {
    Handle* h = static_cast<Handle*>(mh);
    if (!h || n <= 0 || !x || !t || steps < 0 || batch < 128 || batch % 128 != 0 || !(lr > 0)) return PCL_ERR_INVALID;
    MCK(cudaSetDevice(h->device));
    if (n > h->nall_cap) {
        cudaFree(h->Xall); cudaFree(h->Tall);
        h->Xall = h->Tall = nullptr;
        MCK(cudaMalloc(&h->Xall, sizeof(float) * 2 * n));
        MCK(cudaMalloc(&h->Tall, sizeof(float) * n));
        h->nall_cap = n;
    }
    MCK(cudaMemcpyAsync(h->Xall, x, sizeof(float) * 2 * n, cudaMemcpyHostToDevice, h->stream));
    MCK(cudaMemcpyAsync(h->Tall, t, sizeof(float) * n, cudaMemcpyHostToDevice, h->stream));
    h->nall = n;
    int rc = ensure_batch(h, batch);
    if (rc) return rc;
    const long long tail = std::min<long long>(steps, 100);
    MCK(cudaMemsetAsync(h->d_loss, 0, sizeof(double), h->stream));
    const float b1 = 0.9f, b2 = 0.999f;
    for (long long k = 0; k < steps; ++k) {
        k_mlp_gather<<<(batch + 255) / 256, 256, 0, h->stream>>>(h->Xall, h->Tall, n, h->X, h->T, batch,
                                                                 uint32_t(seed), uint32_t(seed >> 32), uint32_t(k));
        MCK(cudaGetLastError());
        if (k == steps - tail) MCK(cudaMemsetAsync(h->d_loss, 0, sizeof(double), h->stream));
        if ((rc = grad_batch(h, batch))) return rc;
        h->adam_t += 1;
        // cosine decay to 5% of lr over the call
        double fr = steps > 1 ? double(k) / double(steps - 1) : 1.0;
        float lrk = float(lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(3.14159265358979 * fr))));
        float c1 = float(1.0 / (1.0 - std::pow(double(b1), double(h->adam_t))));
        float c2 = float(1.0 / (1.0 - std::pow(double(b2), double(h->adam_t))));
        k_mlp_adam<<<(kNParam + 255) / 256, 256, 0, h->stream>>>(h->P, h->G, h->M, h->V, h->W2, h->W3, lrk, b1, b2,
                                                                  1e-8f, c1, c2);
        MCK(cudaGetLastError());
        if ((k & 255) == 255 && (rc = check_err(h))) return rc;
    }
    double l = 0.0;
    MCK(cudaMemcpyAsync(&l, h->d_loss, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    rc = check_err(h);
    if (loss) *loss = tail > 0 ? l / double(tail) : 0.0;
    return rc;
}

}  // extern "C"
