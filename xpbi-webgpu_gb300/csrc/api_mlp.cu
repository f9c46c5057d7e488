// C ABI of the warm-start network (declared in include/xpbi.h): forward,
// gradient and GPU training on host-supplied rows. Not in the reference.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "xpbi.h"
#include "xpbi_internal.h"

namespace xpbi {
int mlp_param_count();
size_t mlp_blob_bytes();
void mlp_pack(const float* dParams, void* dBlob, cudaStream_t st);
cudaError_t mlp_forward(const float* dX, uint32_t rows, const void* dBlob, float* dY, float* dZ, int* dErr,
                        cudaStream_t st, bool skipZero);
cudaError_t mlp_grad(const float* dX, const float* dT, uint32_t rows, const void* dBlob, float* dY, float* dZ,
                     float* dPartial, float* dSq, float* dGrad, float* dLoss, int* dErr, cudaStream_t st);
void mlp_adam(float* dW, const float* dG, float* dM, float* dV, float lr, int step, cudaStream_t st);
int setError(int code, const std::string& msg);
}  // namespace xpbi

using namespace xpbi;

namespace {

// Device allocations of one call, released on scope exit.
struct Scratch {
  std::vector<void*> p;
  ~Scratch() {
    for (void* q : p) cudaFree(q);
  }
  template <class T>
  T* get(size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, n * sizeof(T) > 0 ? n * sizeof(T) : 16) != cudaSuccess) return nullptr;
    p.push_back(q);
    return static_cast<T*>(q);
  }
};

#define MLP_CK(call)                                                                          \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return setError(XPBI_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int deviceErr(int* dErr) {
  int e = 0;
  MLP_CK(cudaMemcpy(&e, dErr, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) return setError(XPBI_ERR_DEVICE, "tensor-core wait expired in the network kernels");
  return XPBI_OK;
}

}  // namespace

extern "C" {

int xpbi_mlp_param_count(void) { return mlp_param_count(); }

int xpbi_mlp_forward(const float* X, uint32_t rows, const float* params, float* y) {
  if (!X || !params || !y) return setError(XPBI_ERR_INVALID, "NULL argument");
  if (rows == 0) return XPBI_OK;
  Scratch s;
  const int P = mlp_param_count();
  float* dX = s.get<float>((size_t)rows * 16);
  float* dP = s.get<float>(P);
  void* dB = s.get<uint8_t>(mlp_blob_bytes());
  float* dY = s.get<float>(rows);
  int* dE = s.get<int>(1);
  if (!dX || !dP || !dB || !dY || !dE) return setError(XPBI_ERR_OOM, "cudaMalloc failed");
  MLP_CK(cudaMemcpy(dX, X, sizeof(float) * rows * 16, cudaMemcpyHostToDevice));
  MLP_CK(cudaMemcpy(dP, params, sizeof(float) * P, cudaMemcpyHostToDevice));
  MLP_CK(cudaMemset(dE, 0, sizeof(int)));
  mlp_pack(dP, dB, 0);
  MLP_CK(mlp_forward(dX, rows, dB, dY, nullptr, dE, 0, false));
  MLP_CK(cudaDeviceSynchronize());
  int rc = deviceErr(dE);
  if (rc) return rc;
  MLP_CK(cudaMemcpy(y, dY, sizeof(float) * rows, cudaMemcpyDeviceToHost));
  return XPBI_OK;
}

int xpbi_mlp_grad(const float* X, const float* T, uint32_t rows, const float* params, float* grad, float* loss) {
  if (!X || !T || !params || !grad) return setError(XPBI_ERR_INVALID, "NULL argument");
  if (rows == 0) return setError(XPBI_ERR_INVALID, "rows must be > 0");
  Scratch s;
  const int P = mlp_param_count();
  const uint32_t tiles = (rows + 127) / 128;
  float* dX = s.get<float>((size_t)rows * 16);
  float* dT = s.get<float>(rows);
  float* dP = s.get<float>(P);
  void* dB = s.get<uint8_t>(mlp_blob_bytes());
  float* dY = s.get<float>(rows);
  float* dZ = s.get<float>((size_t)rows * 64 * 3);
  float* dPart = s.get<float>((size_t)tiles * P);
  float* dSq = s.get<float>(tiles);
  float* dG = s.get<float>(P);
  float* dL = s.get<float>(1);
  int* dE = s.get<int>(1);
  if (!dX || !dT || !dP || !dB || !dY || !dZ || !dPart || !dSq || !dG || !dL || !dE)
    return setError(XPBI_ERR_OOM, "cudaMalloc failed");
  MLP_CK(cudaMemcpy(dX, X, sizeof(float) * rows * 16, cudaMemcpyHostToDevice));
  MLP_CK(cudaMemcpy(dT, T, sizeof(float) * rows, cudaMemcpyHostToDevice));
  MLP_CK(cudaMemcpy(dP, params, sizeof(float) * P, cudaMemcpyHostToDevice));
  MLP_CK(cudaMemset(dE, 0, sizeof(int)));
  mlp_pack(dP, dB, 0);
  MLP_CK(mlp_grad(dX, dT, rows, dB, dY, dZ, dPart, dSq, dG, dL, dE, 0));
  MLP_CK(cudaDeviceSynchronize());
  int rc = deviceErr(dE);
  if (rc) return rc;
  MLP_CK(cudaMemcpy(grad, dG, sizeof(float) * P, cudaMemcpyDeviceToHost));
  if (loss) MLP_CK(cudaMemcpy(loss, dL, sizeof(float), cudaMemcpyDeviceToHost));
  return XPBI_OK;
}

// Adam on the GPU over consecutive mini-batches of (X, T), cycling through
// the rows in the order given (callers shuffle). params is updated in place;
// loss_history (may be NULL) receives each step's batch loss.
int xpbi_mlp_train(const float* X, const float* T, uint32_t rows, float* params, int32_t steps, uint32_t batch,
                   float lr, float* loss_history) {
  if (!X || !T || !params) return setError(XPBI_ERR_INVALID, "NULL argument");
  if (rows == 0 || batch == 0 || steps < 0) return setError(XPBI_ERR_INVALID, "empty training set");
  if (batch > rows) batch = rows;
  Scratch s;
  const int P = mlp_param_count();
  const uint32_t tiles = (batch + 127) / 128;
  float* dX = s.get<float>((size_t)rows * 16);
  float* dT = s.get<float>(rows);
  float* dW = s.get<float>(P);
  float* dM = s.get<float>(P);
  float* dV = s.get<float>(P);
  void* dB = s.get<uint8_t>(mlp_blob_bytes());
  float* dY = s.get<float>(batch);
  float* dZ = s.get<float>((size_t)batch * 64 * 3);
  float* dPart = s.get<float>((size_t)tiles * P);
  float* dSq = s.get<float>(tiles);
  float* dG = s.get<float>(P);
  float* dL = s.get<float>(steps > 0 ? steps : 1);
  int* dE = s.get<int>(1);
  if (!dX || !dT || !dW || !dM || !dV || !dB || !dY || !dZ || !dPart || !dSq || !dG || !dL || !dE)
    return setError(XPBI_ERR_OOM, "cudaMalloc failed");
  MLP_CK(cudaMemcpy(dX, X, sizeof(float) * rows * 16, cudaMemcpyHostToDevice));
  MLP_CK(cudaMemcpy(dT, T, sizeof(float) * rows, cudaMemcpyHostToDevice));
  MLP_CK(cudaMemcpy(dW, params, sizeof(float) * P, cudaMemcpyHostToDevice));
  MLP_CK(cudaMemset(dM, 0, sizeof(float) * P));
  MLP_CK(cudaMemset(dV, 0, sizeof(float) * P));
  MLP_CK(cudaMemset(dE, 0, sizeof(int)));
  uint32_t off = 0;
  for (int t = 0; t < steps; ++t) {
    if (off + batch > rows) off = 0;
    mlp_pack(dW, dB, 0);
    MLP_CK(mlp_grad(dX + (size_t)off * 16, dT + off, batch, dB, dY, dZ, dPart, dSq, dG, dL + t, dE, 0));
    mlp_adam(dW, dG, dM, dV, lr, t + 1, 0);
    off += batch;
  }
  MLP_CK(cudaDeviceSynchronize());
  int rc = deviceErr(dE);
  if (rc) return rc;
  MLP_CK(cudaMemcpy(params, dW, sizeof(float) * P, cudaMemcpyDeviceToHost));
  if (loss_history && steps > 0) MLP_CK(cudaMemcpy(loss_history, dL, sizeof(float) * steps, cudaMemcpyDeviceToHost));
  return XPBI_OK;
}

}  // extern "C"
