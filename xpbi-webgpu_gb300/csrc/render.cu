// Headless particle renderer: the reference's frame (web/js/shaders/render.js,
// drawn by web/js/main.js:232-272 with one sample per pixel and a `less`
// depth test) rasterised by CUDA kernels into a device image, with no
// graphics API.
//
// Every fragment is merged into a 64-bit word per pixel, (depth bits << 32)
// | RGBA8, by atomicMin: depths are non-negative floats, so their bit
// patterns order like the values, and the nearest fragment wins whatever
// the order the threads run in (equal depths keep the smaller colour word).
//   k_background  clear colour, depth 1, and the gridded ground quad
//                 (fsGround, with the screen-space derivative of fwidth
//                 taken from the neighbouring pixel centres' ray hits)
//   k_lines       the 12 edges of the domain box (fsLines), one-pixel DDA
//   k_particles   one thread per particle: the view-space billboard of
//                 vsParticle covers an axis-aligned pixel rectangle; each
//                 pixel centre inside it gets fsParticle's depth-correct
//                 sphere and shading
//   k_resolve     the colour bytes of each pixel
#include <cuda_runtime.h>

#include <cstdint>

#include "render.h"

namespace xpbi {

namespace {

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 norm3(F3 a) { return a * (1.f / sqrtf(dot3(a, a))); }
__device__ __forceinline__ F3 mix3(F3 a, F3 b, float t) { return a + (b - a) * t; }
__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.f), 1.f); }
__device__ __forceinline__ float fractf(float x) { return x - floorf(x); }
__device__ __forceinline__ float smoothstepf(float e0, float e1, float x) {
  const float t = clamp01((x - e0) / (e1 - e0));
  return t * t * (3.f - 2.f * t);
}

// column-major 4x4 times (p, w)
__device__ __forceinline__ void mat4mul(const float* m, float x, float y, float z, float w, float out[4]) {
#pragma unroll
  for (int r = 0; r < 4; ++r) out[r] = m[r] * x + m[4 + r] * y + m[8 + r] * z + m[12 + r] * w;
}
__device__ __forceinline__ F3 viewPoint(const RenderParams& P, F3 p) {
  float o[4];
  mat4mul(P.view, p.x, p.y, p.z, 1.f, o);
  return {o[0], o[1], o[2]};
}
__device__ __forceinline__ F3 viewDir(const RenderParams& P, F3 d) {
  float o[4];
  mat4mul(P.view, d.x, d.y, d.z, 0.f, o);
  return {o[0], o[1], o[2]};
}

__device__ __forceinline__ uint32_t packColor(F3 c) {
  const uint32_t r = (uint32_t)__float2int_rn(clamp01(c.x) * 255.f);
  const uint32_t g = (uint32_t)__float2int_rn(clamp01(c.y) * 255.f);
  const uint32_t b = (uint32_t)__float2int_rn(clamp01(c.z) * 255.f);
  return r | (g << 8) | (b << 16) | (255u << 24);
}
__device__ __forceinline__ unsigned long long packFrag(float depth, uint32_t rgba) {
  return ((unsigned long long)__float_as_uint(depth) << 32) | rgba;
}

// the view-space point where pixel centre (px, py) meets the plane z = zv
__device__ __forceinline__ F3 pixelOnPlane(const RenderParams& P, float px, float py, float zv) {
  const float xn = px / P.width * 2.f - 1.f;
  const float yn = 1.f - py / P.height * 2.f;
  return {xn * (-zv) / P.proj[0], yn * (-zv) / P.proj[5], zv};
}

// world ray hit of pixel centre (px, py) with the ground plane y = groundY
__device__ __forceinline__ bool groundHit(const RenderParams& P, float px, float py, F3& w) {
  const F3 pv = pixelOnPlane(P, px, py, -1.f);  // a point on the view ray
  // view -> world: the view matrix is orthonormal, world = R^T (v - t)
  const F3 rx = f3(P.view[0], P.view[4], P.view[8]);
  const F3 ry = f3(P.view[1], P.view[5], P.view[9]);
  const F3 rz = f3(P.view[2], P.view[6], P.view[10]);
  const F3 dir = f3(rx.x * pv.x + ry.x * pv.y + rz.x * pv.z, rx.y * pv.x + ry.y * pv.y + rz.y * pv.z,
                    rx.z * pv.x + ry.z * pv.y + rz.z * pv.z);
  const F3 eye = f3(P.eye[0], P.eye[1], P.eye[2]);
  if (fabsf(dir.y) < 1e-12f) return false;
  const float t = (P.groundY - eye.y) / dir.y;
  if (!(t > 0.f)) return false;
  w = eye + dir * t;
  return true;
}

__global__ void k_background(RenderParams P, unsigned long long* __restrict__ img) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= (uint32_t)P.width || y >= (uint32_t)P.height) return;
  const F3 bg = f3(0.10f, 0.11f, 0.13f);
  unsigned long long frag = packFrag(1.f, packColor(bg));
  F3 w;
  if (P.drawGround && groundHit(P, x + 0.5f, y + 0.5f, w) && fabsf(w.x - 0.5f) <= 12.f &&
      fabsf(w.z - 0.5f) <= 12.f) {
    float c[4];
    mat4mul(P.viewProj, w.x, w.y, w.z, 1.f, c);
    const float depth = c[2] / c[3];
    if (depth >= 0.f && depth < 1.f) {
      // fwidth(p * 4) from the neighbouring pixel centres
      F3 wx = w, wy = w;
      groundHit(P, x + 1.5f, y + 0.5f, wx);
      groundHit(P, x + 0.5f, y + 1.5f, wy);
      const float fx = fabsf(wx.x - w.x) * 4.f + fabsf(wy.x - w.x) * 4.f;
      const float fz = fabsf(wx.z - w.z) * 4.f + fabsf(wy.z - w.z) * 4.f;
      const float gx = fabsf(fractf(w.x * 4.f - 0.5f) - 0.5f) / fmaxf(fx, 1e-4f);
      const float gz = fabsf(fractf(w.z * 4.f - 0.5f) - 0.5f) / fmaxf(fz, 1e-4f);
      const float line = 1.f - fminf(fminf(gx, gz), 1.f);
      F3 col = mix3(f3(0.16f, 0.17f, 0.20f), f3(0.24f, 0.26f, 0.30f), line * 0.8f);
      const float dx = w.x - 0.5f, dz = w.z - 0.5f;
      const float fade = smoothstepf(1.2f, 5.0f, sqrtf(dx * dx + dz * dz));
      col = mix3(col, bg, fade);
      frag = packFrag(depth, packColor(col));
    }
  }
  img[(size_t)y * P.width + x] = frag;
}

__global__ void k_lines(RenderParams P, unsigned long long* __restrict__ img) {
  const int e = blockIdx.x;  // edge
  if (e >= 12 || !P.drawBox) return;
  const F3 a = f3(P.boxMin[0], P.boxMin[1], P.boxMin[2]), b = f3(P.boxMax[0], P.boxMax[1], P.boxMax[2]);
  const F3 C[8] = {f3(a.x, a.y, a.z), f3(b.x, a.y, a.z), f3(b.x, a.y, b.z), f3(a.x, a.y, b.z),
                   f3(a.x, b.y, a.z), f3(b.x, b.y, a.z), f3(b.x, b.y, b.z), f3(a.x, b.y, b.z)};
  const int E[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
  // clip the edge in view space at the near plane
  F3 v0 = viewPoint(P, C[E[e][0]]), v1 = viewPoint(P, C[E[e][1]]);
  const float zn = -P.nearZ;
  if (v0.z > zn && v1.z > zn) return;
  if (v0.z > zn) v0 = v1 + (v0 - v1) * ((zn - v1.z) / (v0.z - v1.z));
  if (v1.z > zn) v1 = v0 + (v1 - v0) * ((zn - v0.z) / (v1.z - v0.z));
  float c0[4], c1[4];
  mat4mul(P.proj, v0.x, v0.y, v0.z, 1.f, c0);
  mat4mul(P.proj, v1.x, v1.y, v1.z, 1.f, c1);
  const float sx0 = (c0[0] / c0[3] + 1.f) * 0.5f * P.width, sy0 = (1.f - c0[1] / c0[3]) * 0.5f * P.height;
  const float sx1 = (c1[0] / c1[3] + 1.f) * 0.5f * P.width, sy1 = (1.f - c1[1] / c1[3]) * 0.5f * P.height;
  const float len = fmaxf(fabsf(sx1 - sx0), fabsf(sy1 - sy0));
  const int steps = (int)fminf(ceilf(len), 16384.f);
  const uint32_t rgba = packColor(f3(0.45f, 0.48f, 0.55f));
  for (int s = threadIdx.x; s <= steps; s += blockDim.x) {
    const float t = steps > 0 ? (float)s / steps : 0.f;
    const float sx = sx0 + (sx1 - sx0) * t, sy = sy0 + (sy1 - sy0) * t;
    const int px = (int)floorf(sx), py = (int)floorf(sy);
    if (px < 0 || py < 0 || px >= P.width || py >= P.height) continue;
    // perspective-correct depth: interpolate 1/w and z/w
    const float iw = (1.f - t) / c0[3] + t / c1[3];
    const float zw = (1.f - t) * (c0[2] / c0[3]) / c0[3] + t * (c1[2] / c1[3]) / c1[3];
    const float depth = zw / iw;
    if (depth < 0.f || depth >= 1.f) continue;
    atomicMin(img + (size_t)py * P.width + px, packFrag(depth, rgba));
  }
}

__global__ void k_particles(RenderParams P, const float4* __restrict__ pos, const float4* __restrict__ vel,
                            const uint32_t* __restrict__ matWords, uint32_t n, unsigned long long* __restrict__ img) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p4 = pos[i];
  const F3 vc = viewPoint(P, f3(p4.x, p4.y, p4.z));
  const float r = P.particleRadius;
  if (!(vc.z < -P.nearZ)) return;  // billboard behind the near plane
  // vsParticle: material colour with the seeded albedo variation
  const uint32_t mi = min((uint32_t)p4.w, 7u);
  const uint32_t* mw = matWords + mi * 16u;
  const float kind = (float)mw[3];
  F3 base = f3(__uint_as_float(mw[8]), __uint_as_float(mw[9]), __uint_as_float(mw[10]));
  base = base * (0.88f + 0.24f * (fractf(p4.w) * 2.04f));
  const float4 v4 = vel[i];
  const float speed = sqrtf(v4.x * v4.x + v4.y * v4.y + v4.z * v4.z);
  // the billboard's pixel rectangle: corners vc +- r at depth vc.z
  const float sx = P.proj[0] / (-vc.z), sy = P.proj[5] / (-vc.z);
  const float x0 = ((vc.x - r) * sx + 1.f) * 0.5f * P.width, x1 = ((vc.x + r) * sx + 1.f) * 0.5f * P.width;
  const float y0 = (1.f - (vc.y + r) * sy) * 0.5f * P.height, y1 = (1.f - (vc.y - r) * sy) * 0.5f * P.height;
  const int ix0 = max((int)ceilf(x0 - 0.5f), 0), ix1 = min((int)ceilf(x1 - 0.5f), P.width);
  const int iy0 = max((int)ceilf(y0 - 0.5f), 0), iy1 = min((int)ceilf(y1 - 0.5f), P.height);
  if (ix0 >= ix1 || iy0 >= iy1) return;
  if ((int64_t)(ix1 - ix0) * (iy1 - iy0) > (int64_t)P.maxPixelsPerParticle) return;
  const F3 L = norm3(viewDir(P, f3(P.lightDir[0], P.lightDir[1], P.lightDir[2])));
  const F3 up = norm3(viewDir(P, f3(0.f, 1.f, 0.f)));
  const bool water = kind > 5.5f;
  for (int y = iy0; y < iy1; ++y) {
    for (int x = ix0; x < ix1; ++x) {
      const F3 q = pixelOnPlane(P, x + 0.5f, y + 0.5f, vc.z);
      const float u = (q.x - vc.x) / r, v = (q.y - vc.y) / r;
      const float r2 = u * u + v * v;
      if (r2 > 1.f) continue;
      const float nz = sqrtf(1.f - r2);
      const F3 nv = f3(u, v, nz);
      const F3 vp = vc + nv * r;
      float c[4];
      mat4mul(P.proj, vp.x, vp.y, vp.z, 1.f, c);
      const float depth = c[2] / c[3];
      if (depth < 0.f || depth >= 1.f) continue;
      unsigned long long* dst = img + (size_t)y * P.width + x;
      const unsigned long long frag0 = packFrag(depth, 0u);
      if (frag0 >= *dst) continue;  // already behind a nearer fragment
      const float diff = fmaxf(dot3(nv, L), 0.f);
      const float hemi = 0.5f + 0.5f * dot3(nv, up);
      F3 col = base * (0.35f + 0.55f * diff + 0.35f * hemi * 0.5f);
      if (water) {
        const float f1 = 1.f - nz;
        col = mix3(col, f3(0.75f, 0.9f, 1.0f), f1 * f1 * 0.6f);
        col = mix3(col, f3(0.85f, 0.95f, 1.0f), fminf(fmaxf(speed * 0.25f, 0.f), 0.45f));
      }
      const F3 V = norm3(vp * -1.f);
      const F3 H = norm3(L + V);
      const float spec = powf(fmaxf(dot3(nv, H), 0.f), 48.f) * (water ? 0.6f : 0.15f);
      col = col + f3(spec, spec, spec);
      atomicMin(dst, packFrag(depth, packColor(col)));
    }
  }
}

__global__ void k_resolve(const unsigned long long* __restrict__ img, uint32_t count, uint32_t* __restrict__ rgba) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) rgba[i] = (uint32_t)(img[i] & 0xffffffffull);
}

}  // namespace

void render_frame(const RenderParams& P, const float4* pos, const float4* vel, const uint32_t* matWords, uint32_t n,
                  unsigned long long* img, uint32_t* rgba, cudaStream_t st) {
  const dim3 tb(16, 16), gb((P.width + 15) / 16, (P.height + 15) / 16);
  k_background<<<gb, tb, 0, st>>>(P, img);
  k_lines<<<12, 256, 0, st>>>(P, img);
  if (n) k_particles<<<(n + 127) / 128, 128, 0, st>>>(P, pos, vel, matWords, n, img);
  const uint32_t count = (uint32_t)P.width * (uint32_t)P.height;
  k_resolve<<<(count + 255) / 256, 256, 0, st>>>(img, count, rgba);
}

}  // namespace xpbi
