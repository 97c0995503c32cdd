// C ABI of the learned proposal's kernels on caller-owned device buffers.
#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/spray_gpu.h"
#include "mlp.cuh"

namespace spray {
int fail(int code, const std::string& msg);
}

namespace {

using spray::fail;
namespace ml = spray::mlp;
static_assert(sizeof(spray_mlp_sample) == sizeof(ml::Sample), "sample layout");

struct Scope {
  cudaStream_t s = nullptr;
  int* err = nullptr;
  float* partial = nullptr;
  int nsms = 0;
  ~Scope() {
    if (partial) cudaFree(partial);
    if (err) cudaFree(err);
    if (s) cudaStreamDestroy(s);
  }
};

int setup(Scope& sc, int32_t device, int nparts) {
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sc.nsms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sc.s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&sc.err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(sc.err, 0, sizeof(int), sc.s);
  if (e == cudaSuccess && nparts > 0) e = cudaMalloc(&sc.partial, (size_t)nparts * ml::kPartial * sizeof(float));
  if (e != cudaSuccess) return fail(SPRAY_GPU_ECUDA, cudaGetErrorString(e));
  return SPRAY_GPU_OK;
}

int finish(Scope& sc) {
  cudaError_t e = cudaStreamSynchronize(sc.s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return fail(SPRAY_GPU_ECUDA, cudaGetErrorString(e));
  int err = 0;
  e = cudaMemcpy(&err, sc.err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(SPRAY_GPU_ECUDA, cudaGetErrorString(e));
  if (err) return fail(SPRAY_GPU_ETIMEOUT, "a tensor-core wait gave up");
  return SPRAY_GPU_OK;
}

ml::Net net(const float* params, const float* boxes, const float norm[4], int* err) {
  ml::Net n;
  n.params = params;
  n.boxes = boxes;
  for (int c = 0; c < 3; ++c) n.norm.centre[c] = norm[c];
  n.norm.scale = norm[3];
  n.error = err;
  return n;
}

int gradGrid(int nsms, int64_t n) {
  const int64_t tiles = (n + ml::kTile - 1) / ml::kTile;
  return (int)std::max<int64_t>(1, std::min<int64_t>(tiles, ml::gradBlocks(nsms)));
}

}  // namespace

extern "C" {

int32_t spray_mlp_param_count(void) { return ml::kParams; }

int spray_mlp_forward_dev(const float* params, const float* boxes, const float norm[4],
                          const spray_mlp_sample* samples, int64_t n, float* logits, int32_t* pred,
                          int32_t device) {
  if (!params || !boxes || !norm || (n > 0 && (!samples || !logits || !pred)))
    return fail(SPRAY_GPU_EINVAL, "null argument");
  if (n < 0) return fail(SPRAY_GPU_EINVAL, "negative sample count");
  Scope sc;
  if (int r = setup(sc, device, 0)) return r;
  if (n == 0) return SPRAY_GPU_OK;
  const int64_t tiles = (n + ml::kTile - 1) / ml::kTile;
  const int grid = (int)std::min<int64_t>(tiles, 4 * sc.nsms);
  ml::launchPredictSamples(sc.s, net(params, boxes, norm, sc.err), reinterpret_cast<const ml::Sample*>(samples),
                           n, logits, pred, grid);
  return finish(sc);
}

int spray_mlp_grad_dev(const float* params, const float* boxes, const float norm[4],
                       const spray_mlp_sample* samples, int64_t n, float* grad, int32_t device) {
  if (!params || !boxes || !norm || !grad || (n > 0 && !samples)) return fail(SPRAY_GPU_EINVAL, "null argument");
  if (n < 0) return fail(SPRAY_GPU_EINVAL, "negative sample count");
  Scope sc;
  if (int r = setup(sc, device, 0)) return r;
  const int g = gradGrid(sc.nsms, n);
  cudaError_t e = cudaMalloc(&sc.partial, (size_t)g * ml::kPartial * sizeof(float));
  if (e != cudaSuccess) return fail(SPRAY_GPU_ECUDA, cudaGetErrorString(e));
  // labelled rows, counted on the host copy of the labels
  std::vector<spray_mlp_sample> h(n);
  if (n > 0) {
    e = cudaMemcpy(h.data(), samples, (size_t)n * sizeof(spray_mlp_sample), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(SPRAY_GPU_ECUDA, cudaGetErrorString(e));
  }
  int64_t labelled = 0;
  for (auto& q : h) labelled += (q.label >= 0 && q.label < std::min(q.ncand, 8)) ? 1 : 0;
  const float inv = labelled > 0 ? 1.0f / (float)labelled : 0.0f;
  ml::Net nt = net(params, boxes, norm, sc.err);
  ml::launchGrad(sc.s, nt, reinterpret_cast<const ml::Sample*>(samples), n, inv, sc.partial, g);
  ml::launchReduceAdam(sc.s, sc.partial, g, grad, nullptr, nullptr, nullptr, 0.0f, 0);
  return finish(sc);
}

int spray_mlp_train_dev(float* params, float* adam_m, float* adam_v, const float* boxes, const float norm[4],
                        const spray_mlp_sample* samples, int64_t n, int32_t batch, float lr, int32_t steps,
                        int32_t first_step, float* losses, int32_t device) {
  if (!params || !adam_m || !adam_v || !boxes || !norm || !samples) return fail(SPRAY_GPU_EINVAL, "null argument");
  if (n <= 0 || batch <= 0 || steps < 0 || first_step < 1 || !(lr > 0.0f))
    return fail(SPRAY_GPU_EINVAL, "need n > 0, batch > 0, steps >= 0, first_step >= 1, lr > 0");
  Scope sc;
  if (int r = setup(sc, device, 0)) return r;
  const int64_t b = std::min<int64_t>(batch, n);
  const int g = gradGrid(sc.nsms, b);
  float* grad = nullptr;
  cudaError_t e = cudaMalloc(&sc.partial, (size_t)g * ml::kPartial * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&grad, ml::kPartial * sizeof(float));
  if (e != cudaSuccess) {
    if (grad) cudaFree(grad);
    return fail(SPRAY_GPU_ECUDA, cudaGetErrorString(e));
  }
  std::vector<spray_mlp_sample> h(n);
  e = cudaMemcpy(h.data(), samples, (size_t)n * sizeof(spray_mlp_sample), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    cudaFree(grad);
    return fail(SPRAY_GPU_ECUDA, cudaGetErrorString(e));
  }
  ml::Net nt = net(params, boxes, norm, sc.err);
  std::vector<float> lossv(steps, 0.0f);
  int rc = SPRAY_GPU_OK;
  for (int k = 0; k < steps && rc == SPRAY_GPU_OK; ++k) {
    const int64_t start = ((int64_t)k * b) % n;
    const int64_t len = std::min<int64_t>(b, n - start);
    int64_t labelled = 0;
    for (int64_t i = start; i < start + len; ++i)
      labelled += (h[i].label >= 0 && h[i].label < std::min(h[i].ncand, 8)) ? 1 : 0;
    const float inv = labelled > 0 ? 1.0f / (float)labelled : 0.0f;
    ml::launchGrad(sc.s, nt, reinterpret_cast<const ml::Sample*>(samples) + start, len, inv, sc.partial, g);
    ml::launchReduceAdam(sc.s, sc.partial, g, grad, params, adam_m, adam_v, lr, first_step + k);
    if (losses) {
      float tail[2];
      e = cudaMemcpyAsync(tail, grad + ml::kParams, 2 * sizeof(float), cudaMemcpyDeviceToHost, sc.s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(sc.s);
      if (e != cudaSuccess) rc = fail(SPRAY_GPU_ECUDA, cudaGetErrorString(e));
      else lossv[k] = tail[1] > 0.0f ? tail[0] / tail[1] : 0.0f;
    }
  }
  if (rc == SPRAY_GPU_OK) rc = finish(sc);
  cudaFree(grad);
  if (rc == SPRAY_GPU_OK && losses && steps > 0) {
    e = cudaMemcpy(losses, lossv.data(), steps * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(SPRAY_GPU_ECUDA, cudaGetErrorString(e));
  }
  return rc;
}

}  // extern "C"
