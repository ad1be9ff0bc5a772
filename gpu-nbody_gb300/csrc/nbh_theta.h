// nbh_theta.h — learned opening angle: model layout and launchers (nbh_theta.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace nbh {

struct StepParams;

constexpr int kMlpIn = 12;
constexpr int kMlpHid = 64;
constexpr int kMlpParams = kMlpHid * kMlpIn + kMlpHid + kMlpHid * kMlpHid + kMlpHid + kMlpHid + 1;

// Device copy of the installed model: BF16 weight tiles for the tensor cores, FP32 biases
// and the feature normalisation.
struct ThetaDev {
    __nv_bfloat16 w1[kMlpHid * 16];   // W1 padded to 16 inputs
    __nv_bfloat16 w2[kMlpHid * kMlpHid];
    __nv_bfloat16 w3[8 * kMlpHid];    // row 0 = W3, rows 1..7 zero
    float b1[kMlpHid];
    float b2[kMlpHid];
    float b3;
    float mean[kMlpIn];
    float inv_std[kMlpIn];
    float theta_min, theta_max;
};

// Work buffers of the training kernels for a batch of n samples.
struct MlpWork {
    float *H1, *H2, *Y, *dH1, *dH2, *dY;
};

void launch_theta(const StepParams& p, const ThetaDev* mdl, float* theta_out, int grid, cudaStream_t s);
void launch_features(const StepParams& p, const ThetaDev* mdl, const float4* src, const float* theta_prev,
                     float* feat, int grid, cudaStream_t s);
void launch_model_convert(const float* prm, ThetaDev* mdl, cudaStream_t s);

void mlp_grad(const float* prm, const float* X, const float* T, int n, float q, MlpWork& w, float* grad, float* loss,
              cudaStream_t s);
void mlp_forward(const float* prm, const float* X, int n, MlpWork& w, cudaStream_t s);
void adam_step(float* prm, const float* g, float* m1, float* m2, float lr, int t, cudaStream_t s);

}  // namespace nbh
