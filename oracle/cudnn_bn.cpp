// cuDNN batch normalisation as the reference's normaliser calls it -- a test
// oracle for the library's normalize_kernel.
//
// TEST INFRASTRUCTURE ONLY: tests/ load this through ctypes to check the
// library's z-score against the arithmetic the reference actually runs; the
// product never links it.
//
// normalizer::normalize (src/include/normalizer.cu:71-113) z-scores a host
// array of reads x length samples by running cudnnBatchNormalizationForwardTraining
// in place: NCHW tensor (1, C = reads, H = length, W = 1), mode
// CUDNN_BATCHNORM_SPATIAL (one mean and variance per read), alpha 1, beta 0,
// scale 1 and bias 0 per channel (normalizer.cu:26-27, :50-56),
// exponentialAverageFactor 1 / (1 + length), no running statistics and
// epsilon 1e-4 (normalizer.cu:98-100).  This file makes the same call on a
// device buffer the caller owns.
#include <cudnn.h>

#include <cstdio>

extern "C" {

// Text of the last failure.
static char g_err[256];
const char *cudnn_bn_last_error(void) { return g_err; }

// In place on d_x (reads x length floats, read-major).  d_scale / d_bias hold
// `reads` floats (1 and 0 for the reference's call).  Runs on the legacy
// default stream; the caller synchronises.  Returns 0 or the cuDNN status.
int cudnn_bn_normalize(float *d_x, int reads, int length, const float *d_scale, const float *d_bias,
                       double epsilon) {
  cudnnHandle_t h = nullptr;
  cudnnTensorDescriptor_t x_desc = nullptr, bn_desc = nullptr;
  const float alpha = 1.f, beta = 0.f;
  cudnnStatus_t st = cudnnCreate(&h);
  if (st == CUDNN_STATUS_SUCCESS) st = cudnnCreateTensorDescriptor(&x_desc);
  if (st == CUDNN_STATUS_SUCCESS) st = cudnnCreateTensorDescriptor(&bn_desc);
  if (st == CUDNN_STATUS_SUCCESS)
    st = cudnnSetTensor4dDescriptor(x_desc, CUDNN_TENSOR_NCHW, CUDNN_DATA_FLOAT, 1, reads, length, 1);
  if (st == CUDNN_STATUS_SUCCESS) st = cudnnDeriveBNTensorDescriptor(bn_desc, x_desc, CUDNN_BATCHNORM_SPATIAL);
  if (st == CUDNN_STATUS_SUCCESS)
    st = cudnnBatchNormalizationForwardTraining(h, CUDNN_BATCHNORM_SPATIAL, &alpha, &beta, x_desc, d_x, x_desc,
                                                d_x, bn_desc, d_scale, d_bias, 1.0 / (1.0 + length), nullptr,
                                                nullptr, epsilon, nullptr, nullptr);
  if (st != CUDNN_STATUS_SUCCESS) snprintf(g_err, sizeof(g_err), "%s", cudnnGetErrorString(st));
  if (bn_desc) cudnnDestroyTensorDescriptor(bn_desc);
  if (x_desc) cudnnDestroyTensorDescriptor(x_desc);
  if (h) cudnnDestroy(h);
  return (int)st;
}

int cudnn_bn_version(void) { return (int)cudnnGetVersion(); }

}  // extern "C"
