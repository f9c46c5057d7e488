// The warm-start network: a per-particle MLP 16 -> 64 -> 64 -> 64 -> 1 with
// SiLU activations, BF16 weights and FP32 accumulation, run on the tcgen05
// tensor cores (operands in shared memory, accumulators in TMEM).
//
// A CTA of 128 threads owns a tile of 128 rows (one row per thread, TMEM
// lane = row), so each layer is one M=128, N=64 MMA chain (K = 16 or 64 in
// steps of 16) followed by an epilogue in which every thread reads its own
// row back from TMEM, adds the bias, applies SiLU and writes the bf16 row
// of the next layer's A tile. The 64 -> 1 output layer is a per-thread dot
// product in FP32.
//
// Training (hand-written backward):
//   forward stores the pre-activations z1..z3 (f32) and the output;
//   backward forms dy = 2 (y - t) / B, dz3 = (dy w4) * silu'(z3), and the
//   activation gradients dh2 = dz3 W3, dh1 = dz2 W2 on the tensor cores
//   (A = bf16 dz, B = W^T tiles); weight gradients dW = dz^T h are FP32
//   SIMT reductions over the CTA's rows into per-CTA partials, summed in a
//   fixed order afterwards; Adam updates FP32 master weights, which are then
//   repacked as BF16 tiles.
//
// Every mbarrier wait is bounded; on expiry the kernel raises an error bit,
// stops issuing work and still releases its TMEM.
#include <cuda_bf16.h>

#include "tc.cuh"
#include "xpbi_internal.h"

namespace xpbi {

namespace {

constexpr int kRows = 128;
constexpr int kIn = 16;
constexpr int kHid = 64;
constexpr uint32_t kSpin = 1u << 24;
constexpr int kErrMma = 2;

// Parameter vector (f32 master): W1[64][16] b1[64] W2[64][64] b2 W3[64][64] b3 w4[64] b4
constexpr int oW1 = 0, oB1 = oW1 + kHid * kIn, oW2 = oB1 + kHid, oB2 = oW2 + kHid * kHid, oW3 = oB2 + kHid,
              oB3 = oW3 + kHid * kHid, oW4 = oB3 + kHid, oB4 = oW4 + kHid, kParams = oB4 + 1;
static_assert(kParams == 9473, "parameter count");

// Packed blob (device): bf16 core-layout tiles, then f32 vectors.
constexpr uint32_t bW1 = 0;                          // 64 x 16 bf16  = 2 KB
constexpr uint32_t bW2 = bW1 + kHid * kIn * 2;       // 64 x 64       = 8 KB
constexpr uint32_t bW3 = bW2 + kHid * kHid * 2;      // 64 x 64
constexpr uint32_t bW2T = bW3 + kHid * kHid * 2;     // W2 transposed
constexpr uint32_t bW3T = bW2T + kHid * kHid * 2;    // W3 transposed
constexpr uint32_t bF32 = bW3T + kHid * kHid * 2;    // b1 b2 b3 w4(bf16-rounded) b4 as f32
constexpr uint32_t kBlobBytes = bF32 + (4 * kHid + 4) * 4;
// shared-memory image of the forward kernel: A tile, W1, W2, W3, f32 vectors
constexpr uint32_t sA = 0;                           // 128 x 64 bf16 = 16 KB
constexpr uint32_t sW1 = sA + kRows * kHid * 2;
constexpr uint32_t sW2 = sW1 + kHid * kIn * 2;
constexpr uint32_t sW3 = sW2 + kHid * kHid * 2;
constexpr uint32_t sF32 = sW3 + kHid * kHid * 2;
constexpr uint32_t kFwdSmem = sF32 + (4 * kHid + 4) * 4;

// SiLU z * sigmoid(z) with the MUFU exponential and reciprocal (a few ulp)
__device__ __forceinline__ float sigm(float z) { return __fdividef(1.f, 1.f + __expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
// SiLU for inference: z sigmoid(z) = h + h tanh(h) with h = z / 2 and the
// MUFU tanh (one special-function op instead of an exponential and a
// reciprocal). Its ~5e-4 relative error lies below the bf16 rounding every
// activation gets; training keeps the exact form its backward pass uses.
__device__ __forceinline__ float tanhMufu(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float siluFast(float z) {
  const float h = 0.5f * z;
  return fmaf(h, tanhMufu(h), h);
}
__device__ __forceinline__ float dsilu(float z) {
  const float s = sigm(z);
  return s * (1.f + z * (1.f - s));
}

// f32 params -> packed blob
__global__ void k_mlp_pack(const float* __restrict__ p, uint8_t* __restrict__ blob) {
  for (int t = threadIdx.x; t < kHid * kHid; t += blockDim.x) {
    const int r = t / kHid, k = t % kHid;  // W[out=r][in=k]
    *reinterpret_cast<__nv_bfloat16*>(blob + bW2 + tc::coreOffset(r, k, kHid)) = __float2bfloat16_rn(p[oW2 + t]);
    *reinterpret_cast<__nv_bfloat16*>(blob + bW3 + tc::coreOffset(r, k, kHid)) = __float2bfloat16_rn(p[oW3 + t]);
    // transposed tiles: row = in, col = out
    *reinterpret_cast<__nv_bfloat16*>(blob + bW2T + tc::coreOffset(k, r, kHid)) = __float2bfloat16_rn(p[oW2 + t]);
    *reinterpret_cast<__nv_bfloat16*>(blob + bW3T + tc::coreOffset(k, r, kHid)) = __float2bfloat16_rn(p[oW3 + t]);
  }
  for (int t = threadIdx.x; t < kHid * kIn; t += blockDim.x) {
    const int r = t / kIn, k = t % kIn;
    *reinterpret_cast<__nv_bfloat16*>(blob + bW1 + tc::coreOffset(r, k, kIn)) = __float2bfloat16_rn(p[oW1 + t]);
  }
  float* f = reinterpret_cast<float*>(blob + bF32);
  for (int t = threadIdx.x; t < kHid; t += blockDim.x) {
    f[t] = p[oB1 + t];
    f[kHid + t] = p[oB2 + t];
    f[2 * kHid + t] = p[oB3 + t];
    f[3 * kHid + t] = __bfloat162float(__float2bfloat16_rn(p[oW4 + t]));
  }
  if (threadIdx.x == 0) f[4 * kHid] = p[oB4];
}

struct FwdOut {
  float* y;        // [rows] network output
  float* z;        // [3][rows][64] pre-activations (training) or null
};

// Forward over `rows` feature rows X[rows][16] (f32).
__global__ void __launch_bounds__(kRows) k_mlp_fwd(const float* __restrict__ X, uint32_t rows,
                                                   const uint8_t* __restrict__ blob, FwdOut out, int* err,
                                                   int skipZero) {
  extern __shared__ __align__(1024) uint8_t sm[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  const int tid = threadIdx.x, warp = tid >> 5;
  const bool infer = out.z == nullptr;  // no pre-activations kept: inference
  // weights -> shared memory (straight copy of the packed tiles)
  {
    const uint4* src = reinterpret_cast<const uint4*>(blob);
    uint4* dst = reinterpret_cast<uint4*>(sm + sW1);
    for (uint32_t q = tid; q < (bW2T - bW1) / 16u; q += kRows) dst[q] = src[q];  // W1, W2, W3
    const float* fs = reinterpret_cast<const float*>(blob + bF32);
    float* fd = reinterpret_cast<float*>(sm + sF32);
    for (uint32_t q = tid; q < 4 * kHid + 1; q += kRows) fd[q] = fs[q];
  }
  if (warp == 0) tc::tmemAlloc(&tbase, 64);
  if (tid == 0) tc::mbarInit(&bar, 1);
  tc::fenceBeforeSync();
  __syncthreads();
  tc::fenceAfterSync();
  const uint32_t tmem = tbase;
  const uint32_t tRow = tmem + ((uint32_t)(warp * 32) << 16);
  const float* F = reinterpret_cast<const float*>(sm + sF32);
  const uint32_t aAddr = tc::smemAddr(sm + sA), w1Addr = tc::smemAddr(sm + sW1), w2Addr = tc::smemAddr(sm + sW2),
                 w3Addr = tc::smemAddr(sm + sW3);
  constexpr uint32_t idesc = tc::idescBf16F32(kRows, kHid);
  uint32_t phase = 0;
  bool ok = true;
  const uint32_t ntiles = (rows + kRows - 1) / kRows;
  for (uint32_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const uint32_t row = tile * kRows + tid;
    // ---- layer 1 input: features as bf16, K = 16
    bool active = false;
    {
      float x[kIn];
      if (row < rows) {
        const float4* xr = reinterpret_cast<const float4*>(X + (size_t)row * kIn);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float4 v = __ldg(xr + q);
          x[4 * q] = v.x; x[4 * q + 1] = v.y; x[4 * q + 2] = v.z; x[4 * q + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int q = 0; q < kIn; ++q) x[q] = 0.f;
      }
#pragma unroll
      for (int q = 0; q < kIn; ++q) active |= x[q] != 0.f;
#pragma unroll
      for (int c = 0; c < kIn / 8; ++c) {
        __align__(16) __nv_bfloat16 h[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) h[e] = __float2bfloat16_rn(x[8 * c + e]);
        *reinterpret_cast<uint4*>(sm + sA + tc::coreOffset(tid, 8 * c, kIn)) = *reinterpret_cast<uint4*>(h);
      }
    }
    // the solver's tiles of water particles (all-zero feature rows) need no
    // prediction: their output is defined as 0
    if (skipZero && !__syncthreads_or(active)) {
      if (row < rows) out.y[row] = 0.f;
      continue;
    }
    float y = F[4 * kHid];
    for (int layer = 0; layer < 3 && ok; ++layer) {
      tc::fenceProxyAsync();
      tc::fenceBeforeSync();
      __syncthreads();  // A written by every thread; every warp done with the accumulator
      if (tid == 0) {
        tc::fenceAfterSync();
        const uint32_t K = layer == 0 ? kIn : kHid;
        const uint32_t wAddr = layer == 0 ? w1Addr : (layer == 1 ? w2Addr : w3Addr);
        const uint32_t sbo = (K / 8) * 128;
        for (uint32_t ks = 0; ks < K / 16; ++ks)
          tc::mma(tmem, tc::smemDesc(aAddr + ks * 256, 128, sbo), tc::smemDesc(wAddr + ks * 256, 128, sbo), idesc,
                  ks > 0);
        tc::commit(&bar);
      }
      if (!tc::mbarWait(&bar, phase, kSpin)) {
        if (tid == 0) atomicOr(err, kErrMma);
        ok = false;
      }
      phase ^= 1u;
      tc::fenceAfterSync();
      // epilogue, 16 columns of this thread's row at a time; the MMA that read
      // A has completed, so the next layer's A row is written in place
      const float* bias = F + layer * kHid;
      const float* w4 = F + 3 * kHid;
#pragma unroll 1
      for (int c = 0; c < kHid / 16; ++c) {
        float z[16];
        tc::ld16(tRow + 16 * c, z);
#pragma unroll
        for (int j = 0; j < 16; ++j) z[j] += bias[16 * c + j];
        if (out.z != nullptr && row < rows) {
          float4* zr = reinterpret_cast<float4*>(out.z + ((size_t)layer * rows + row) * kHid + 16 * c);
#pragma unroll
          for (int q = 0; q < 4; ++q) zr[q] = make_float4(z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
        }
        if (layer < 2) {
#pragma unroll
          for (int h8 = 0; h8 < 2; ++h8) {
            __align__(16) __nv_bfloat16 h[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
              const float a = z[8 * h8 + e];
              h[e] = __float2bfloat16_rn(infer ? siluFast(a) : silu(a));
            }
            *reinterpret_cast<uint4*>(sm + sA + tc::coreOffset(tid, 16 * c + 8 * h8, kHid)) =
                *reinterpret_cast<uint4*>(h);
          }
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) y += (infer ? siluFast(z[j]) : silu(z[j])) * w4[16 * c + j];
        }
      }
    }
    if (ok && row < rows) out.y[row] = y;
  }
  tc::fenceBeforeSync();
  __syncthreads();
  tc::fenceAfterSync();
  if (warp == 0) tc::tmemDealloc(tmem, 64);
}

// Backward over one batch: per-CTA weight-gradient partials and the squared
// error. Shared memory: A tile (bf16 dz, 16 KB), W3T, W2T (8 KB each), the
// CTA's dz and h rows in f32 (2 x 32 KB) and the f32 vectors.
constexpr uint32_t bA = 0;
constexpr uint32_t bW3Ts = bA + kRows * kHid * 2;
constexpr uint32_t bW2Ts = bW3Ts + kHid * kHid * 2;
constexpr uint32_t bDZ = bW2Ts + kHid * kHid * 2;     // f32 [128][64]
constexpr uint32_t bH = bDZ + kRows * kHid * 4;       // f32 [128][64]
constexpr uint32_t bFv = bH + kRows * kHid * 4;
constexpr uint32_t bRed = bFv + (4 * kHid + 4) * 4;   // f32 [128] scratch
constexpr uint32_t kBwdSmem = bRed + kRows * 4;

// SIMT weight-gradient partial: G[j][i] = sum_r dz[r][j] * h[r][i] over the
// CTA's valid rows (h has `nin` columns, stride kHid).
__device__ __forceinline__ void wgradPartial(const float* dz, const float* h, int nin, int nvalid, float* outW,
                                             float* outB) {
  for (int p = threadIdx.x; p < kHid * nin; p += kRows) {
    const int j = p / nin, i = p % nin;
    float acc = 0.f;
    for (int r = 0; r < nvalid; ++r) acc += dz[r * kHid + j] * h[r * kHid + i];
    outW[p] = acc;
  }
  for (int j = threadIdx.x; j < kHid; j += kRows) {
    float acc = 0.f;
    for (int r = 0; r < nvalid; ++r) acc += dz[r * kHid + j];
    outB[j] = acc;
  }
}

__global__ void __launch_bounds__(kRows) k_mlp_bwd(const float* __restrict__ X, const float* __restrict__ T,
                                                   uint32_t rows, const uint8_t* __restrict__ blob,
                                                   const float* __restrict__ Y, const float* __restrict__ Z,
                                                   float* __restrict__ partial, float* __restrict__ sqerr, int* err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  const int tid = threadIdx.x, warp = tid >> 5;
  {
    const uint4* src = reinterpret_cast<const uint4*>(blob + bW2T);
    uint4* d3 = reinterpret_cast<uint4*>(sm + bW3Ts);
    uint4* d2 = reinterpret_cast<uint4*>(sm + bW2Ts);
    const uint32_t n = kHid * kHid * 2 / 16;
    for (uint32_t q = tid; q < n; q += kRows) {
      d2[q] = src[q];       // W2T
      d3[q] = src[n + q];   // W3T
    }
    const float* fs = reinterpret_cast<const float*>(blob + bF32);
    float* fd = reinterpret_cast<float*>(sm + bFv);
    for (uint32_t q = tid; q < 4 * kHid + 1; q += kRows) fd[q] = fs[q];
  }
  if (warp == 0) tc::tmemAlloc(&tbase, 64);
  if (tid == 0) tc::mbarInit(&bar, 1);
  tc::fenceBeforeSync();
  __syncthreads();
  tc::fenceAfterSync();
  const uint32_t tmem = tbase;
  const uint32_t tRow = tmem + ((uint32_t)(warp * 32) << 16);
  const float* Fv = reinterpret_cast<const float*>(sm + bFv);
  float* dz = reinterpret_cast<float*>(sm + bDZ);
  float* h = reinterpret_cast<float*>(sm + bH);
  float* red = reinterpret_cast<float*>(sm + bRed);
  const uint32_t aAddr = tc::smemAddr(sm + bA);
  constexpr uint32_t idesc = tc::idescBf16F32(kRows, kHid);
  const uint32_t tile = blockIdx.x;
  const uint32_t row = tile * kRows + tid;
  const bool valid = row < rows;
  const int nvalid = (int)min((uint32_t)kRows, rows - tile * kRows);
  float* P = partial + (size_t)blockIdx.x * kParams;
  auto zAt = [&](int layer, int j) { return valid ? Z[((size_t)layer * rows + row) * kHid + j] : 0.f; };
  // dy and the squared error
  float dy = 0.f;
  if (valid) {
    const float e = Y[row] - T[row];
    dy = 2.f * e / (float)rows;
    red[tid] = e * e;
  } else {
    red[tid] = 0.f;
  }
  // h3 (f32) and dz3
  float dzr[kHid];
  {
    const float* w4 = Fv + 3 * kHid;
#pragma unroll 4
    for (int j = 0; j < kHid; ++j) {
      const float z3 = zAt(2, j);
      h[tid * kHid + j] = valid ? silu(z3) : 0.f;
      dzr[j] = valid ? dy * w4[j] * dsilu(z3) : 0.f;
    }
  }
  __syncthreads();
  // w4, b4 gradients
  for (int j = tid; j < kHid; j += kRows) {
    float acc = 0.f;
    for (int r = 0; r < nvalid; ++r) {
      const float e = Y[tile * kRows + r] - T[tile * kRows + r];
      acc += 2.f * e / (float)rows * h[r * kHid + j];
    }
    P[oW4 + j] = acc;
  }
  if (tid == 0) {
    float acc = 0.f, se = 0.f;
    for (int r = 0; r < nvalid; ++r) {
      acc += 2.f * (Y[tile * kRows + r] - T[tile * kRows + r]) / (float)rows;
      se += red[r];
    }
    P[oB4] = acc;
    sqerr[blockIdx.x] = se;
  }
  bool ok = true;
  // layers 3 and 2: dz (f32) -> dW, db; dh_prev = dz W (tensor cores); dz_prev
  for (int layer = 2; layer >= 1 && ok; --layer) {
    __syncthreads();
#pragma unroll 4
    for (int j = 0; j < kHid; ++j) {
      dz[tid * kHid + j] = dzr[j];
      h[tid * kHid + j] = valid ? __bfloat162float(__float2bfloat16_rn(silu(zAt(layer - 1, j)))) : 0.f;
    }
#pragma unroll
    for (int c = 0; c < kHid / 8; ++c) {
      __align__(16) __nv_bfloat16 hb[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) hb[e] = __float2bfloat16_rn(dzr[8 * c + e]);
      *reinterpret_cast<uint4*>(sm + bA + tc::coreOffset(tid, 8 * c, kHid)) = *reinterpret_cast<uint4*>(hb);
    }
    tc::fenceProxyAsync();
    tc::fenceBeforeSync();
    __syncthreads();
    if (tid == 0) {
      tc::fenceAfterSync();
      const uint32_t wAddr = tc::smemAddr(sm + (layer == 2 ? bW3Ts : bW2Ts));
      for (uint32_t ks = 0; ks < kHid / 16; ++ks)
        tc::mma(tmem, tc::smemDesc(aAddr + ks * 256, 128, 1024), tc::smemDesc(wAddr + ks * 256, 128, 1024), idesc,
                ks > 0);
      tc::commit(&bar);
    }
    const int oW = layer == 2 ? oW3 : oW2, oB = layer == 2 ? oB3 : oB2;
    wgradPartial(dz, h, kHid, nvalid, P + oW, P + oB);
    if (!tc::mbarWait(&bar, (uint32_t)(2 - layer), kSpin)) {
      if (tid == 0) atomicOr(err, kErrMma);
      ok = false;
    }
    tc::fenceAfterSync();
    float dh[kHid];
#pragma unroll
    for (int c = 0; c < kHid / 16; ++c) tc::ld16(tRow + 16 * c, dh + 16 * c);
#pragma unroll 4
    for (int j = 0; j < kHid; ++j) dzr[j] = valid ? dh[j] * dsilu(zAt(layer - 1, j)) : 0.f;
    tc::fenceBeforeSync();
    __syncthreads();
  }
  // layer 1: dW1 = dz1^T x (x as bf16, the network's input precision)
  __syncthreads();
  for (int j = 0; j < kHid; ++j) dz[tid * kHid + j] = dzr[j];
  for (int k = 0; k < kIn; ++k)
    h[tid * kHid + k] = valid ? __bfloat162float(__float2bfloat16_rn(X[(size_t)row * kIn + k])) : 0.f;
  __syncthreads();
  wgradPartial(dz, h, kIn, nvalid, P + oW1, P + oB1);
  tc::fenceBeforeSync();
  __syncthreads();
  tc::fenceAfterSync();
  if (warp == 0) tc::tmemDealloc(tmem, 64);
}

// grad[p] = sum over CTAs of partial[cta][p] (fixed order); loss likewise.
__global__ void k_mlp_reduce(const float* __restrict__ partial, uint32_t nparts, const float* __restrict__ sqerr,
                             uint32_t rows, float* __restrict__ grad, float* __restrict__ loss) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < (uint32_t)kParams) {
    float acc = 0.f;
    for (uint32_t c = 0; c < nparts; ++c) acc += partial[(size_t)c * kParams + p];
    grad[p] = acc;
  }
  if (p == 0) {
    float se = 0.f;
    for (uint32_t c = 0; c < nparts; ++c) se += sqerr[c];
    *loss = se / (float)rows;
  }
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  const float gi = g[p];
  const float mi = b1 * m[p] + (1.f - b1) * gi;
  const float vi = b2 * v[p] + (1.f - b2) * gi * gi;
  m[p] = mi;
  v[p] = vi;
  w[p] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace

int mlp_param_count() { return kParams; }
size_t mlp_blob_bytes() { return kBlobBytes; }

void mlp_pack(const float* dParams, void* dBlob, cudaStream_t st) {
  k_mlp_pack<<<1, 256, 0, st>>>(dParams, static_cast<uint8_t*>(dBlob));
}

cudaError_t mlp_forward(const float* dX, uint32_t rows, const void* dBlob, float* dY, float* dZ, int* dErr,
                        cudaStream_t st, bool skipZero) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwdSmem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  if (rows == 0) return cudaSuccess;
  const uint32_t ntiles = (rows + kRows - 1) / kRows;
  // 48 registers and 37 KB of shared memory: six CTAs per SM (384 TMEM columns)
  const uint32_t grid = ntiles < 152u * 6u ? ntiles : 152u * 6u;
  k_mlp_fwd<<<grid, kRows, kFwdSmem, st>>>(dX, rows, static_cast<const uint8_t*>(dBlob), FwdOut{dY, dZ}, dErr,
                                           skipZero ? 1 : 0);
  return cudaGetLastError();
}

// One training step's gradient (and mean squared error) on rows X, targets T.
// Scratch: dY [rows], dZ [3 rows 64], dPartial [ceil(rows/128) * params],
// dSq [ceil(rows/128)].
cudaError_t mlp_grad(const float* dX, const float* dT, uint32_t rows, const void* dBlob, float* dY, float* dZ,
                     float* dPartial, float* dSq, float* dGrad, float* dLoss, int* dErr, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, kBwdSmem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  cudaError_t e = mlp_forward(dX, rows, dBlob, dY, dZ, dErr, st);
  if (e != cudaSuccess || rows == 0) return e;
  const uint32_t ntiles = (rows + kRows - 1) / kRows;
  k_mlp_bwd<<<ntiles, kRows, kBwdSmem, st>>>(dX, dT, rows, static_cast<const uint8_t*>(dBlob), dY, dZ, dPartial,
                                            dSq, dErr);
  k_mlp_reduce<<<(kParams + 255) / 256, 256, 0, st>>>(dPartial, ntiles, dSq, rows, dGrad, dLoss);
  return cudaGetLastError();
}

void mlp_adam(float* dW, const float* dG, float* dM, float* dV, float lr, int step, cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<(kParams + 255) / 256, 256, 0, st>>>(dW, dG, dM, dV, lr, b1, b2, 1e-8f, c1, c2);
}

}  // namespace xpbi
