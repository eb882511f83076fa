// Optimisation-step kernels of the batched and served paths: the MSE loss
// gradient of a rendered image against its target, and an Adam update over
// a parameter arena.  Both read every scalar they need from device memory
// (the Adam step count lives on the device), so a CUDA graph can replay them
// step after step without host involvement.
#include "dvg_internal.h"

namespace {

// d_image = scale * (image - target);  loss += sum((image - target)^2)
__global__ void k_mse_grad(const float4 *image, const float4 *target, long long n4, float scale, float4 *d_image,
                           float *loss) {
  float acc = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x) {
    float4 a = image[i], b = target[i];
    float4 d = make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
    acc += d.x * d.x + d.y * d.y + d.z * d.z + d.w * d.w;
    d_image[i] = make_float4(scale * d.x, scale * d.y, scale * d.z, scale * d.w);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ float red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    if (loss) atomicAdd(loss, s);
  }
}

// Adam (Kingma & Ba) with bias correction; lr_scale[i] scales the step of
// element i (0 freezes it).  t = *step + 1.
__global__ void k_adam(float *p, const float *g, float *m, float *v, const float *lr_scale, long long n, float lr,
                       float b1, float b2, float eps, const int *step) {
  int t = *step + 1;
  float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float s = lr_scale ? lr_scale[i] : 1.f;
    if (s == 0.f) continue;
    float gi = g[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= s * lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void k_step_inc(int *step) { *step += 1; }

}  // namespace

extern "C" int dvg_mse_grad(const float *image, const float *target, int64_t num_pixels, float scale, float *d_image,
                            float *loss, void *stream) {
  dvg::clear_error();
  if (!image || !target || !d_image || num_pixels < 0)
    return dvg::fail(DVG_ERR_INVALID, "image, target and d_image must be set");
  if ((reinterpret_cast<uintptr_t>(image) | reinterpret_cast<uintptr_t>(target) | reinterpret_cast<uintptr_t>(d_image)) & 15u)
    return dvg::fail(DVG_ERR_INVALID, "image buffers must be 16-byte aligned");
  if (num_pixels == 0) return DVG_OK;
  long long blocks = (num_pixels + 255) / 256;
  if (blocks > 1024) blocks = 1024;
  k_mse_grad<<<(unsigned)blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const float4 *>(image), reinterpret_cast<const float4 *>(target), num_pixels, scale,
      reinterpret_cast<float4 *>(d_image), loss);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DVG_OK : dvg::cuda_fail(e, "mse gradient launch");
}

extern "C" int dvg_adam_step(float *params, const float *grads, float *m, float *v, const float *lr_scale, int64_t n,
                             float lr, float beta1, float beta2, float eps, int *step, void *stream) {
  dvg::clear_error();
  if (!params || !grads || !m || !v || !step || n < 0)
    return dvg::fail(DVG_ERR_INVALID, "params, grads, moments and step must be set");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (n > 0) {
    long long blocks = (n + 255) / 256;
    if (blocks > 2048) blocks = 2048;
    k_adam<<<(unsigned)blocks, 256, 0, s>>>(params, grads, m, v, lr_scale, n, lr, beta1, beta2, eps, step);
  }
  k_step_inc<<<1, 1, 0, s>>>(step);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DVG_OK : dvg::cuda_fail(e, "adam launch");
}
