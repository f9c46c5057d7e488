// Scene sampling on the device: the lattice samplers of web/js/scenes.js:7-38
// (sampleBox, sampleSphere) for scenes too large to sample on the host.
//
// The lattice is the reference's, point for point: a box's points at cell
// centres lo + (i + 0.5) h for i < max(1, Math.round(extent / h)) per axis, a
// sphere's at c - r + i h for i <= ceil(2 r / h) kept where
// Math.hypot(p - c) <= r; points are numbered in the reference's loop order
// (z outer, x inner; a sphere's kept points compacted in that order), shapes
// one after another. Every coordinate is formed in f64 with one rounding per
// operation (no fused multiply-adds), like the JavaScript numbers, and the
// sphere test evaluates Math.hypot as V8 does (magnitudes scaled by the
// largest, squares summed with Kahan compensation, sqrt(sum) * max), so the
// points equal the host sampler's (scenes.py) bit for bit. The reference
// jitters each coordinate by (Math.random() - 0.5) * jitter * h; here the
// uniforms come from a counter-based generator (Philox-4x32-10, Salmon et al.,
// SC'11) keyed by the seed and counted by the particle's number, so any
// particle's jitter is computed independently of the others.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "xpbi.h"

namespace xpbi {
int setError(int code, const std::string& msg);
}  // namespace xpbi

using namespace xpbi;

namespace {

constexpr int kThreads = 256;

// ---- Philox-4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers:
// as easy as 1, 2, 3", SC 2011): ten rounds of two 32x32->64 multiplies and a
// Feistel-like mix, the key bumped by the Weyl constants between rounds.
__host__ __device__ inline void philoxRound(uint32_t c[4], const uint32_t k[2]) {
  const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
  const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
  const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
  const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
  const uint32_t n0 = hi1 ^ c[1] ^ k[0], n2 = hi0 ^ c[3] ^ k[1];
  c[0] = n0;
  c[1] = lo1;
  c[2] = n2;
  c[3] = lo0;
}
__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  uint32_t k[2] = {k0, k1};
  for (int r = 0; r < 10; ++r) {
    philoxRound(c, k);
    k[0] += 0x9E3779B9u;
    k[1] += 0xBB67AE85u;
  }
}
// A double in [0, 1) from two words: 27 + 26 high bits, as NumPy forms its
// doubles from 32-bit draws.
__device__ __forceinline__ double unitDouble(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// f64 arithmetic with one rounding per operation
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// Math.hypot(a, b, c) as V8 evaluates it
__device__ __forceinline__ double jsHypot3(double a, double b, double c) {
  const double v[3] = {fabs(a), fabs(b), fabs(c)};
  const double m = fmax(fmax(v[0], v[1]), v[2]);
  if (m == 0.0) return 0.0;
  double total = 0.0, comp = 0.0;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const double n = __ddiv_rn(v[q], m);
    const double summand = dsub(dmul(n, n), comp);
    const double prelim = dadd(total, summand);
    comp = dsub(dsub(prelim, total), summand);
    total = prelim;
  }
  return dmul(__dsqrt_rn(total), m);
}

struct ShapeDev {
  int kind;
  int n[3];            // lattice points per axis (sphere: n + 1 each)
  double base[3];      // box: lo; sphere: c - r
  double off;          // box: 0.5 (cell centres); sphere: 0
  double centre[3], radius;
  double jitterH;      // jitter * h
  uint32_t mat, first; // material, number of the shape's first particle
  float state0;
};

__device__ __forceinline__ void latticePoint(const ShapeDev& s, double h, uint64_t l, double p[3]) {
  const uint64_t i = l % (uint64_t)s.n[0], jk = l / (uint64_t)s.n[0];
  const uint64_t j = jk % (uint64_t)s.n[1], k = jk / (uint64_t)s.n[1];
  const double idx[3] = {(double)i, (double)j, (double)k};
#pragma unroll
  for (int a = 0; a < 3; ++a) p[a] = dadd(s.base[a], dmul(dadd(idx[a], s.off), h));
}

__device__ __forceinline__ bool inSphere(const ShapeDev& s, const double p[3]) {
  return jsHypot3(dsub(p[0], s.centre[0]), dsub(p[1], s.centre[1]), dsub(p[2], s.centre[2])) <= s.radius;
}

// sphere lattice: kept points per block (block b covers points b*256 ..)
__global__ void k_sphere_count(ShapeDev s, double h, uint64_t points, uint32_t* blockCount) {
  const uint64_t l = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  bool keep = false;
  if (l < points) {
    double p[3];
    latticePoint(s, h, l, p);
    keep = inSphere(s, p);
  }
  const uint32_t c = __syncthreads_count(keep);
  if (threadIdx.x == 0) blockCount[blockIdx.x] = c;
}

// the kept points compacted in lattice order: lattice index of each
__global__ void k_sphere_compact(ShapeDev s, double h, uint64_t points, const uint32_t* __restrict__ blockStart,
                                 uint64_t* __restrict__ keptLattice) {
  __shared__ uint32_t warpCount[kThreads / 32];
  const uint64_t l = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  bool keep = false;
  if (l < points) {
    double p[3];
    latticePoint(s, h, l, p);
    keep = inSphere(s, p);
  }
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const unsigned m = __ballot_sync(0xffffffffu, keep);
  if (lane == 0) warpCount[warp] = (uint32_t)__popc(m);
  __syncthreads();
  uint32_t before = blockStart[blockIdx.x];
  for (unsigned w = 0; w < warp; ++w) before += warpCount[w];
  if (keep) keptLattice[before + (uint32_t)__popc(m & ((1u << lane) - 1u))] = l;
}

// particle q of a shape: its lattice point (a sphere's from the compaction)
// plus the jitter, rounded to f32
__global__ void k_fill(ShapeDev s, double h, uint32_t count, const uint64_t* __restrict__ keptLattice, uint32_t k0,
                       uint32_t k1, float* __restrict__ pos, uint32_t* __restrict__ mat, float* __restrict__ st) {
  const uint32_t q = blockIdx.x * kThreads + threadIdx.x;
  if (q >= count) return;
  const uint64_t l = keptLattice ? keptLattice[q] : (uint64_t)q;
  double p[3];
  latticePoint(s, h, l, p);
  const uint32_t id = s.first + q;
  uint32_t c0[4] = {id, 0u, 0u, 0u}, c1[4] = {id, 1u, 0u, 0u};
  philox4x32_10(c0, k0, k1);
  philox4x32_10(c1, k0, k1);
  const double u[3] = {unitDouble(c0[0], c0[1]), unitDouble(c0[2], c0[3]), unitDouble(c1[0], c1[1])};
  const size_t o = 3 * (size_t)id;
#pragma unroll
  for (int a = 0; a < 3; ++a) pos[o + a] = __double2float_rn(dadd(p[a], dmul(dsub(u[a], 0.5), s.jitterH)));
  mat[id] = s.mat;
  st[id] = s.state0;
}

int jsRound(double x) { return (int)std::floor(x + 0.5); }  // Math.round: halves toward +infinity

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

extern "C" int xpbi_philox4x32_10(const uint32_t counter[4], const uint32_t key[2], uint32_t out[4]) {
  if (!counter || !key || !out) return setError(XPBI_ERR_INVALID, "NULL argument");
  uint32_t c[4] = {counter[0], counter[1], counter[2], counter[3]};
  philox4x32_10(c, key[0], key[1]);
  std::memcpy(out, c, sizeof(c));
  return XPBI_OK;
}

extern "C" int xpbi_sample_shapes(const xpbi_shape* shapes, uint32_t n_shapes, double h, uint64_t seed,
                                  uint32_t capacity, float* positions, uint32_t* mat_ids, float* states,
                                  uint32_t* count) {
  if (!shapes || !count || n_shapes == 0) return setError(XPBI_ERR_INVALID, "shapes and count are required");
  if (!(h > 0) || !std::isfinite(h)) return setError(XPBI_ERR_INVALID, "h must be positive and finite");
  std::vector<ShapeDev> sd(n_shapes);
  std::vector<uint64_t> points(n_shapes);
  for (uint32_t q = 0; q < n_shapes; ++q) {
    const xpbi_shape& in = shapes[q];
    ShapeDev& s = sd[q];
    std::memset(&s, 0, sizeof(s));
    s.kind = in.kind;
    s.mat = in.mat_id;
    s.state0 = in.state0;
    if (!(in.jitter >= 0) || !std::isfinite(in.jitter)) return setError(XPBI_ERR_INVALID, "jitter must be >= 0");
    s.jitterH = in.jitter * h;
    if (in.kind == XPBI_SHAPE_BOX) {  // scenes.js:7-20
      for (int a = 0; a < 3; ++a) {
        if (!std::isfinite(in.lo[a]) || !std::isfinite(in.hi[a]))
          return setError(XPBI_ERR_INVALID, "box corners must be finite");
        if (!(in.hi[a] >= in.lo[a])) return setError(XPBI_ERR_INVALID, "box hi must not be below lo");
        const double e = (in.hi[a] - in.lo[a]) / h;
        if (e > 1e6) return setError(XPBI_ERR_INVALID, "box lattice too large");
        s.n[a] = std::max(1, jsRound(e));
        s.base[a] = in.lo[a];
      }
      s.off = 0.5;
    } else if (in.kind == XPBI_SHAPE_SPHERE) {  // scenes.js:22-38
      if (!(in.radius > 0) || !std::isfinite(in.radius)) return setError(XPBI_ERR_INVALID, "radius must be > 0");
      for (int a = 0; a < 3; ++a)
        if (!std::isfinite(in.centre[a])) return setError(XPBI_ERR_INVALID, "sphere centre must be finite");
      const double nn = std::ceil(2 * in.radius / h);
      if (nn > 1e5) return setError(XPBI_ERR_INVALID, "sphere lattice too large");
      for (int a = 0; a < 3; ++a) {
        s.n[a] = (int)nn + 1;
        s.base[a] = in.centre[a] - in.radius;
        s.centre[a] = in.centre[a];
      }
      s.radius = in.radius;
    } else {
      return setError(XPBI_ERR_INVALID, "shape kind must be XPBI_SHAPE_BOX or XPBI_SHAPE_SPHERE");
    }
    points[q] = (uint64_t)s.n[0] * s.n[1] * s.n[2];
    if (points[q] > 0xffffffffull) return setError(XPBI_ERR_INVALID, "shape lattice has more than 2^32 points");
  }
  // counts: a box keeps every lattice point, a sphere those inside (device)
  std::vector<uint32_t> kept(n_shapes);
  std::vector<DevBuf> blockStarts(n_shapes);
  uint64_t total = 0;
  for (uint32_t q = 0; q < n_shapes; ++q) {
    if (sd[q].kind == XPBI_SHAPE_BOX) {
      kept[q] = (uint32_t)points[q];
    } else {
      const uint64_t blocks = (points[q] + kThreads - 1) / kThreads;
      DevBuf cnt;
      if (cudaMalloc(&cnt.p, sizeof(uint32_t) * blocks) != cudaSuccess ||
          cudaMalloc(&blockStarts[q].p, sizeof(uint32_t) * blocks) != cudaSuccess)
        return setError(XPBI_ERR_OOM, "xpbi_sample_shapes: device memory");
      k_sphere_count<<<(unsigned)blocks, kThreads>>>(sd[q], h, points[q], (uint32_t*)cnt.p);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return setError(XPBI_ERR_CUDA, std::string("sphere count: ") + cudaGetErrorString(e));
      std::vector<uint32_t> c(blocks);
      e = cudaMemcpy(c.data(), cnt.p, sizeof(uint32_t) * blocks, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return setError(XPBI_ERR_CUDA, std::string("sphere count: ") + cudaGetErrorString(e));
      uint32_t run = 0;
      for (uint64_t b = 0; b < blocks; ++b) {
        const uint32_t x = c[b];
        c[b] = run;
        run += x;
      }
      e = cudaMemcpy(blockStarts[q].p, c.data(), sizeof(uint32_t) * blocks, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return setError(XPBI_ERR_CUDA, std::string("sphere scan: ") + cudaGetErrorString(e));
      kept[q] = run;
    }
    sd[q].first = (uint32_t)total;
    total += kept[q];
    if (total > 0x7fffffffull) return setError(XPBI_ERR_INVALID, "more than 2^31 particles");
  }
  *count = (uint32_t)total;
  if (!positions) return XPBI_OK;  // sizing call
  if (total > capacity) return setError(XPBI_ERR_INVALID, "capacity below the sampled particle count");
  if (total == 0) return XPBI_OK;
  DevBuf pos, mat, st;
  if (cudaMalloc(&pos.p, 12 * total) != cudaSuccess || cudaMalloc(&mat.p, 4 * total) != cudaSuccess ||
      cudaMalloc(&st.p, 4 * total) != cudaSuccess)
    return setError(XPBI_ERR_OOM, "xpbi_sample_shapes: device memory");
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (uint32_t q = 0; q < n_shapes; ++q) {
    if (kept[q] == 0) continue;
    DevBuf lat;
    if (sd[q].kind == XPBI_SHAPE_SPHERE) {
      const uint64_t blocks = (points[q] + kThreads - 1) / kThreads;
      if (cudaMalloc(&lat.p, sizeof(uint64_t) * kept[q]) != cudaSuccess)
        return setError(XPBI_ERR_OOM, "xpbi_sample_shapes: device memory");
      k_sphere_compact<<<(unsigned)blocks, kThreads>>>(sd[q], h, points[q], (const uint32_t*)blockStarts[q].p,
                                                       (uint64_t*)lat.p);
    }
    k_fill<<<(kept[q] + kThreads - 1) / kThreads, kThreads>>>(sd[q], h, kept[q], (const uint64_t*)lat.p, k0, k1,
                                                             (float*)pos.p, (uint32_t*)mat.p, (float*)st.p);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();  // before `lat` is freed
    if (e != cudaSuccess) return setError(XPBI_ERR_CUDA, std::string("sampling: ") + cudaGetErrorString(e));
  }
  cudaError_t e = cudaMemcpy(positions, pos.p, 12 * total, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && mat_ids) e = cudaMemcpy(mat_ids, mat.p, 4 * total, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && states) e = cudaMemcpy(states, st.p, 4 * total, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return setError(XPBI_ERR_CUDA, std::string("sample read-back: ") + cudaGetErrorString(e));
  return XPBI_OK;
}
