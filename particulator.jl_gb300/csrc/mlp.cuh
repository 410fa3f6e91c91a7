// The learned inverse-CDF sampler network shared by the training kernels,
// the batched inference kernel and the step's learned mode:
//   (a, b) -> 128 -> 128 -> 128 -> 1, GELU after every hidden layer,
// a = (log10(T / eV) - 6) / 2 over T in [1e4, 1e8] eV, b = 2u - 1.
// The two 128 x 128 layers run on the tensor cores (BF16 operands, FP32
// accumulators in tensor memory); the 2 -> 128 and 128 -> 1 layers are FP32.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace pcl {
namespace mlp {

constexpr int kH = 128;
// FP32 parameter block layout
constexpr int oW1 = 0;                // [128][2]
constexpr int ob1 = oW1 + 2 * kH;     // [128]
constexpr int oW2 = ob1 + kH;         // [128 out][128 in]
constexpr int ob2 = oW2 + kH * kH;
constexpr int oW3 = ob2 + kH;
constexpr int ob3 = oW3 + kH * kH;
constexpr int ow4 = ob3 + kH;         // [128]
constexpr int ob4 = ow4 + kH;         // [1]
constexpr int kNParam = ob4 + 1;

// Device view of one network: FP32 master parameters and the BF16 copies of
// the two tensor-core layers ([out][in], row-major).
struct Net {
    const float* P;
    const __nv_bfloat16* W2;
    const __nv_bfloat16* W3;
};

// Activations kept by the training forward pass for the backward kernels.
struct TrainBuf {
    float* z1; float* z2; float* z3;              // pre-activations [n][128]
    __nv_bfloat16* h1; __nv_bfloat16* h2;         // GEMM inputs [n][128]
    __nv_bfloat16* dz2; __nv_bfloat16* dz3;       // GEMM inputs of the backward pass
};

// Shared memory of the kernels (bytes, dynamic)
constexpr int kTileBytes = kH * kH * 2;

__global__ void k_mlp_forward(Net net, const float* X, long long n, float* Y, TrainBuf tb, const float* T,
                              float* G, double* loss, int* err);
__global__ void k_mlp_bwd_a(Net net, const float* X, long long n, TrainBuf tb, float* G, int* err);
__global__ void k_mlp_bwd_w(long long n, TrainBuf tb, float* G, int* err);
__global__ void k_mlp_adam(float* P, const float* G, float* M, float* V, __nv_bfloat16* W2, __nv_bfloat16* W3,
                           float lr, float b1, float b2, float eps, float c1, float c2);
__global__ void k_mlp_sync_bf16(const float* P, __nv_bfloat16* W2, __nv_bfloat16* W3);
__global__ void k_mlp_gather(const float* Xall, const float* Tall, long long nall, float* X, float* T, int B,
                             uint32_t key0, uint32_t key1, uint32_t step);

// Several networks evaluated on the same inputs in one launch (blockIdx.y =
// network): the step's learned round.
constexpr int kMaxNets = 8;
struct NetSet {
    Net net[kMaxNets];
    float* Y[kMaxNets];
};
constexpr int kInferThreads = 512;   // 4 column quarters x 128 rows
__global__ void k_mlp_infer(NetSet ns, const float* X, long long cap, const unsigned long long* n_dev, int* err);

constexpr size_t kFwdSmem = 3 * kTileBytes + 1024 + 3 * kH * 4 + 64;
constexpr size_t kInferSmem = 3 * kTileBytes + 1024 + 4 * kH * 4 + 64;
constexpr size_t kBwdASmem = 3 * kTileBytes + 1024 + 4 * kH * 4 + 64;
constexpr size_t kBwdWSmem = 4 * kTileBytes + 1024 + 64;

}  // namespace mlp
}  // namespace pcl
