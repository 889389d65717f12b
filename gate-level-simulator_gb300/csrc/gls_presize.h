// Learned presize of gate-output lists: features, the MLP inference kernels
// (BF16 tcgen05 and an FP32 CUDA-core twin) and the training kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "gls_internal.h"

namespace gls {

constexpr int kIn = 32, kHid = 128;
constexpr int kOffW1 = 0, kOffB1 = kHid * kIn, kOffW2 = kOffB1 + kHid, kOffB2 = kOffW2 + kHid * kHid,
              kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid, kParams = kOffB3 + 1;

// Shared-memory image of the BF16 weights in the tcgen05 canonical K-major
// layout without swizzle: element (row r, k) of an R x K operand sits at byte
//   (r / 8) * (K / 8) * 128 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// i.e. 8-row x 16-byte core matrices, K-adjacent core matrices 128 bytes
// apart (leading byte offset) and 8-row groups (K / 8) * 128 bytes apart
// (stride byte offset).
constexpr uint32_t kImgW1 = 0, kImgW2 = kHid * kIn * 2, kImgBytes = kImgW2 + kHid * kHid * 2;
__host__ __device__ inline uint32_t canon_off(uint32_t r, uint32_t k, uint32_t K)
{
    return (r >> 3) * (K >> 3) * 128u + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

struct PresizeArgs {
    // rows: either host-supplied feature rows, or gate outputs [lo, lo + n)
    // whose features are the static row plus the input-net lengths
    const float *rows;            // n x 32, or null
    const WinDev *wv;             // windows (blockIdx.y) supplying net_len, saif, pred, err; or null
    uint32_t nwin;
    const float *feat_static;     // per driver x 32
    const DrvMeta *meta;
    const uint8_t *lut;           // cell truth tables
    const uint32_t *net_len;
    const unsigned long long *saif;   // T0 / T1 / TX per net (input nets are complete)
    uint32_t lo, n;
    const float *params;          // FP32 parameters (CUDA-core kernel; biases and w3 for both)
    const uint4 *img;             // BF16 weight image (tensor-core kernel)
    float margin;
    uint32_t slack;
    uint32_t *pred;               // per row: reserved events, or null
    float *y;                     // per row: network output, or null
    uint32_t *err;                // set on a tensor-core wait timeout
};

void prepare_presize_kernels();
void launch_presize(const PresizeArgs &a, bool tensor_cores, cudaStream_t st);
void launch_features(const PresizeArgs &a, float *out, cudaStream_t st);

}  // namespace gls
