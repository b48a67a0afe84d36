// Learned field surrogate: constants, the network's parameter layout and the
// device-side feature map shared by the training and inference kernels.
//
// Network (one per cone): input p = (x, y, z, a) in octree units and scale
// factor, normalised to u = (p - lo) * sc - 1 in [-1, 1]^4; 64 Fourier
// features s_j = F_j . u (F holds pi times the frequencies), giving
// h0 = [sin s_0..63, cos s_0..63] (128); four hidden layers
// h_l = silu(W_l h_(l-1) + b_l) of width 128; the output layer gives the
// normalised field y = W_5 h_4 + b_5, read as (phi, dphidx, dphidy, dphidz,
// dphidt) = y * std + mean.  W_l is row-major [out][in].  The output layer is
// padded to 16 rows (the tensor-core N) whose extra rows stay zero.
#pragma once
#include <cstdint>

namespace mpf {
namespace surr {

constexpr int kFreq = 64;
constexpr int kWidth = 128;
constexpr int kHidden = 4;
constexpr int kOut = 5;
constexpr int kOutPad = 16;
constexpr int kLayerStride = kWidth * kWidth + kWidth;   // W then b of a hidden layer
constexpr int kW5 = kHidden * kLayerStride;              // output weights [16][128]
constexpr int kB5 = kW5 + kOutPad * kWidth;              // output bias [16]
constexpr int kParams = kB5 + kOutPad;

// Inference image of the parameters (bytes): BF16 weight tiles in the
// tensor-core operand layout (mpf_umma.cuh), FP32 biases (those of the hidden
// layers halved: the activation is formed from z / 2).
constexpr int kPackW5 = kHidden * kWidth * kWidth * 2;
constexpr int kPackB = kPackW5 + kOutPad * kWidth * 2;
constexpr int kPackB5 = kPackB + kHidden * kWidth * 4;
constexpr int kPackBytes = kPackB5 + kOutPad * 4;

struct Spec {
    float lo[4], sc[4];        // input normalisation
    float freq[kFreq][4];      // pi * frequencies
    float mean[kOut], stdv[kOut];
};

// the sampling domain: a square cone about +x from the observer
struct Cone {
    double tan_y, tan_z, r_min, r_max;
};

__host__ __device__ __forceinline__ void normalise(const Spec& S, const float* p, float* u)
{
#pragma unroll
    for (int d = 0; d < 4; ++d) u[d] = (p[d] - S.lo[d]) * S.sc[d] - 1.f;
}

__host__ __device__ __forceinline__ float project(const Spec& S, int j, const float* u)
{
    return S.freq[j][0] * u[0] + S.freq[j][1] * u[1] + S.freq[j][2] * u[2] + S.freq[j][3] * u[3];
}

}  // namespace surr
}  // namespace mpf
