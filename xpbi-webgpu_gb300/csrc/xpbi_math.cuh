// Device math of the XPBI substep: SPH kernels, grid helpers, 3x3 SVD,
// StVK-Hencky and the five return mappings. Restates the math of
// web/js/shaders/common.js (cited per function) in f32 with the same
// operation order, so results track the WGSL to rounding.
#pragma once
#include "xpbi_internal.h"

namespace xpbi {

// ----------------------------------------------------------------- vectors
struct V3 {
  float x, y, z;
  __device__ __forceinline__ float& operator[](int k) { return k == 0 ? x : (k == 1 ? y : z); }
  __device__ __forceinline__ float operator[](int k) const { return k == 0 ? x : (k == 1 ? y : z); }
};
__device__ __forceinline__ V3 v3(float a, float b, float c) { return V3{a, b, c}; }
__device__ __forceinline__ V3 splat(float s) { return V3{s, s, s}; }
__device__ __forceinline__ V3 xyz(const float4& a) { return V3{a.x, a.y, a.z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float length(V3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ V3 normalize(V3 a) { return a / length(a); }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
__device__ __forceinline__ V3 vclamp(V3 v, float lo, float hi) {
  return {clampf(v.x, lo, hi), clampf(v.y, lo, hi), clampf(v.z, lo, hi)};
}
__device__ __forceinline__ V3 vmaxs(V3 v, float m) { return {fmaxf(v.x, m), fmaxf(v.y, m), fmaxf(v.z, m)}; }
__device__ __forceinline__ V3 vlog(V3 v) { return {logf(v.x), logf(v.y), logf(v.z)}; }
__device__ __forceinline__ V3 vexp(V3 v) { return {expf(v.x), expf(v.y), expf(v.z)}; }
__device__ __forceinline__ V3 vsqrt(V3 v) { return {sqrtf(v.x), sqrtf(v.y), sqrtf(v.z)}; }

// Column-major 3x3, c[j] = column j (WGSL mat3x3f).
struct M3 {
  V3 c[3];
};
__device__ __forceinline__ M3 mzero() { return {{splat(0.f), splat(0.f), splat(0.f)}}; }
__device__ __forceinline__ M3 mident() { return {{v3(1.f, 0.f, 0.f), v3(0.f, 1.f, 0.f), v3(0.f, 0.f, 1.f)}}; }
__device__ __forceinline__ V3 mul(const M3& A, V3 v) { return A.c[0] * v.x + A.c[1] * v.y + A.c[2] * v.z; }
__device__ __forceinline__ M3 mul(const M3& A, const M3& B) {
  return {{mul(A, B.c[0]), mul(A, B.c[1]), mul(A, B.c[2])}};
}
__device__ __forceinline__ M3 transpose(const M3& A) {
  return {{v3(A.c[0].x, A.c[1].x, A.c[2].x), v3(A.c[0].y, A.c[1].y, A.c[2].y),
           v3(A.c[0].z, A.c[1].z, A.c[2].z)}};
}
__device__ __forceinline__ M3 madd(const M3& A, const M3& B) {
  return {{A.c[0] + B.c[0], A.c[1] + B.c[1], A.c[2] + B.c[2]}};
}
__device__ __forceinline__ M3 mscale(const M3& A, float s) { return {{A.c[0] * s, A.c[1] * s, A.c[2] * s}}; }
__device__ __forceinline__ float det(const M3& A) { return dot(A.c[0], cross(A.c[1], A.c[2])); }

// Plane-major 3x3 storage: entry (col c, row r) of particle i at [(3c+r)*N + i].
__device__ __forceinline__ M3 loadM(const float* __restrict__ P, uint32_t N, uint32_t i) {
  M3 m;
#pragma unroll
  for (int c = 0; c < 3; ++c)
    m.c[c] = v3(P[(3 * c + 0) * (size_t)N + i], P[(3 * c + 1) * (size_t)N + i], P[(3 * c + 2) * (size_t)N + i]);
  return m;
}
__device__ __forceinline__ void storeM(float* __restrict__ P, uint32_t N, uint32_t i, const M3& m) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    P[(3 * c + 0) * (size_t)N + i] = m.c[c].x;
    P[(3 * c + 1) * (size_t)N + i] = m.c[c].y;
    P[(3 * c + 2) * (size_t)N + i] = m.c[c].z;
  }
}

// ----------------------------------------------------------------- SPH kernels
// Wendland C2, support 2h (common.js:63-79). sigW is the precomputed
// 21/(16 pi h^3).
__device__ __forceinline__ float kernelW(const SceneDev& S, float r) {
  float q = r / S.h;
  if (q >= 2.f) return 0.f;
  float t = 1.f - 0.5f * q;
  return S.sigW * t * t * t * t * (2.f * q + 1.f);
}
__device__ __forceinline__ V3 kernelGradW(const SceneDev& S, V3 dxv) {
  float r = length(dxv);
  float q = r / S.h;
  if (q >= 2.f || r < 1e-9f) return splat(0.f);
  float t = 1.f - 0.5f * q;
  float dwdq = S.sigW * (-5.f * q) * t * t * t;
  return dxv * (dwdq / (S.h * r));
}
// PBF kernels with H = support (common.js:81-94).
__device__ __forceinline__ float kernelPoly6(const SceneDev& S, float r) {
  float H = S.support;
  if (r >= H) return 0.f;
  float x = H * H - r * r;
  return S.poly6C * x * x * x;
}
__device__ __forceinline__ V3 kernelSpikyGrad(const SceneDev& S, V3 dxv) {
  float H = S.support;
  float r = length(dxv);
  if (r >= H || r < 1e-9f) return splat(0.f);
  float t = H - r;
  return dxv * (S.spikyC * t * t / r);
}

// Same kernels with the square root and the divisions by h and r replaced
// by one reciprocal square root and multiplications by the precomputed 1/h:
// a few ulp from the WGSL expressions, far below the parity tolerance.
// r < 1e-9 (the reference's zero-distance guard) is r^2 < 1e-18.
__device__ __forceinline__ V3 gradWFast(const SceneDev& S, V3 dxv) {
  const float r2 = dot(dxv, dxv);
  if (r2 < 1e-18f) return splat(0.f);
  const float rinv = rsqrtf(r2);
  const float q = r2 * rinv * S.invH;
  if (q >= 2.f) return splat(0.f);
  const float t = 1.f - 0.5f * q;
  const float dwdq = S.sigW * (-5.f * q) * t * t * t;
  return dxv * (dwdq * S.invH * rinv);
}
__device__ __forceinline__ float kernelWFast(const SceneDev& S, float r2) {
  const float q = r2 > 0.f ? r2 * rsqrtf(r2) * S.invH : 0.f;
  if (q >= 2.f) return 0.f;
  const float t = 1.f - 0.5f * q;
  return S.sigW * t * t * t * t * (2.f * q + 1.f);
}
// poly6 from the squared distance: H^2 - r^2 with r^2 taken directly
__device__ __forceinline__ float poly6Fast(const SceneDev& S, float r2) {
  if (r2 >= S.support2) return 0.f;
  const float x = S.support2 - r2;
  return S.poly6C * x * x * x;
}
__device__ __forceinline__ V3 spikyGradFast(const SceneDev& S, V3 dxv, float r2) {
  if (r2 < 1e-18f) return splat(0.f);
  const float rinv = rsqrtf(r2);
  const float r = r2 * rinv;
  if (r >= S.support) return splat(0.f);
  const float t = S.support - r;
  return dxv * (S.spikyC * t * t * rinv);
}

// ----------------------------------------------------------------- grid
// common.js:97-103. Saturating f32->i32 (NaN -> 0) before clamping.
__device__ __forceinline__ int axisCell(float p, float o, float cs, int dim) {
  float fl = floorf((p - o) / cs);
  fl = fminf(fmaxf(fl, 0.f), (float)(dim - 1));
  return (int)fl;
}
struct I3 {
  int x, y, z;
};
__device__ __forceinline__ I3 cellCoord(const SceneDev& S, V3 p) {
  return I3{axisCell(p.x, S.origin[0], S.cs, S.dims[0]), axisCell(p.y, S.origin[1], S.cs, S.dims[1]),
            axisCell(p.z, S.origin[2], S.cs, S.dims[2])};
}
__device__ __forceinline__ uint32_t cellIndex(const SceneDev& S, int x, int y, int z) {
  return (uint32_t)x + (uint32_t)y * (uint32_t)S.dims[0] + (uint32_t)z * (uint32_t)(S.dims[0] * S.dims[1]);
}

// ----------------------------------------------------------------- svd3
// Jacobi eigen-decomposition of F^T F, 6 sweeps (common.js:105-184).
template <int p, int q>
__device__ __forceinline__ void jacobiRot(M3& S, M3& V) {
  float Spq = S.c[q][p];
  float Spp = S.c[p][p];
  float Sqq = S.c[q][q];
  if (fabsf(Spq) < 1e-12f) return;
  float tau = (Sqq - Spp) / (2.f * Spq);
  float t;
  if (tau >= 0.f) t = 1.f / (tau + sqrtf(1.f + tau * tau));
  else t = 1.f / (tau - sqrtf(1.f + tau * tau));
  float c = 1.f / sqrtf(1.f + t * t);
  float s = t * c;
  M3 Sn = S;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float Skp = S.c[p][k], Skq = S.c[q][k];
    Sn.c[p][k] = c * Skp - s * Skq;
    Sn.c[q][k] = s * Skp + c * Skq;
  }
  M3 S2 = Sn;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float Spk = Sn.c[k][p], Sqk = Sn.c[k][q];
    S2.c[k][p] = c * Spk - s * Sqk;
    S2.c[k][q] = s * Spk + c * Sqk;
  }
  S = S2;
  M3 Vn = V;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float Vkp = V.c[p][k], Vkq = V.c[q][k];
    Vn.c[p][k] = c * Vkp - s * Vkq;
    Vn.c[q][k] = s * Vkp + c * Vkq;
  }
  V = Vn;
}

struct SVD {
  M3 U;
  V3 sig;
  M3 V;
};

__device__ __forceinline__ void swapf(float& a, float& b) { float t = a; a = b; b = t; }
__device__ __forceinline__ void swapv(V3& a, V3& b) { V3 t = a; a = b; b = t; }

__device__ __forceinline__ SVD svd3(const M3& F) {
  M3 S = mul(transpose(F), F);
  M3 V = mident();
#pragma unroll 1
  for (int sweep = 0; sweep < 6; ++sweep) {
    jacobiRot<0, 1>(S, V);
    jacobiRot<0, 2>(S, V);
    jacobiRot<1, 2>(S, V);
  }
  V3 sig = v3(sqrtf(fmaxf(S.c[0].x, 0.f)), sqrtf(fmaxf(S.c[1].y, 0.f)), sqrtf(fmaxf(S.c[2].z, 0.f)));
  V3 a0 = V.c[0], a1 = V.c[1], a2 = V.c[2];
  if (sig.x < sig.y) { swapf(sig.x, sig.y); swapv(a0, a1); }
  if (sig.x < sig.z) { swapf(sig.x, sig.z); swapv(a0, a2); }
  if (sig.y < sig.z) { swapf(sig.y, sig.z); swapv(a1, a2); }
  if (dot(cross(a0, a1), a2) < 0.f) a2 = -a2;
  SVD out;
  out.V = {{a0, a1, a2}};
  V3 u0, u1;
  const float eps = 1e-8f;
  if (sig.x > eps) u0 = normalize(mul(F, a0));
  else u0 = v3(1.f, 0.f, 0.f);
  if (sig.y > eps) {
    V3 Fv1 = mul(F, a1);
    u1 = Fv1 - dot(Fv1, u0) * u0;
    float l = length(u1);
    if (l > eps) u1 = u1 / l;
    else u1 = normalize(cross(v3(0.f, 1.f, 0.f), u0) + splat(1e-4f));
  } else {
    V3 a = cross(u0, v3(0.f, 1.f, 0.f));
    if (length(a) < 1e-4f) a = cross(u0, v3(1.f, 0.f, 0.f));
    u1 = normalize(a);
  }
  V3 u2 = cross(u0, u1);
  if (det(F) < 0.f) sig.z = -sig.z;
  out.U = {{u0, u1, u2}};
  out.sig = sig;
  return out;
}

// The same Jacobi sweeps with approximate reciprocal, reciprocal square
// root and division (MUFU based). Rotation angles differ from the IEEE
// version by a few ulp; the decomposition converges to the same U, sigma, V
// to ~1e-6 and the products used downstream (U diag V^T) agree to rounding.
template <int p, int q>
__device__ __forceinline__ void jacobiRotFast(M3& S, M3& V) {
  const float Spq = S.c[q][p];
  const float Spp = S.c[p][p];
  const float Sqq = S.c[q][q];
  if (fabsf(Spq) < 1e-12f) return;
  const float tau = __fdividef(Sqq - Spp, 2.f * Spq);
  const float h2 = 1.f + tau * tau;
  const float root = h2 * rsqrtf(h2);
  const float t = __fdividef(1.f, tau >= 0.f ? tau + root : tau - root);
  const float c = rsqrtf(1.f + t * t);
  const float s = t * c;
  M3 Sn = S;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float Skp = S.c[p][k], Skq = S.c[q][k];
    Sn.c[p][k] = c * Skp - s * Skq;
    Sn.c[q][k] = s * Skp + c * Skq;
  }
  M3 S2 = Sn;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float Spk = Sn.c[k][p], Sqk = Sn.c[k][q];
    S2.c[k][p] = c * Spk - s * Sqk;
    S2.c[k][q] = s * Spk + c * Sqk;
  }
  S = S2;
  M3 Vn = V;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float Vkp = V.c[p][k], Vkq = V.c[q][k];
    Vn.c[p][k] = c * Vkp - s * Vkq;
    Vn.c[q][k] = s * Vkp + c * Vkq;
  }
  V = Vn;
}

__device__ __forceinline__ V3 normalizeFast(V3 a) { return a * rsqrtf(dot(a, a)); }

__device__ __forceinline__ SVD svd3Fast(const M3& F) {
  M3 S = mul(transpose(F), F);
  M3 V = mident();
#pragma unroll 1
  for (int sweep = 0; sweep < 6; ++sweep) {
    jacobiRotFast<0, 1>(S, V);
    jacobiRotFast<0, 2>(S, V);
    jacobiRotFast<1, 2>(S, V);
  }
  V3 sig = v3(sqrtf(fmaxf(S.c[0].x, 0.f)), sqrtf(fmaxf(S.c[1].y, 0.f)), sqrtf(fmaxf(S.c[2].z, 0.f)));
  V3 a0 = V.c[0], a1 = V.c[1], a2 = V.c[2];
  if (sig.x < sig.y) { swapf(sig.x, sig.y); swapv(a0, a1); }
  if (sig.x < sig.z) { swapf(sig.x, sig.z); swapv(a0, a2); }
  if (sig.y < sig.z) { swapf(sig.y, sig.z); swapv(a1, a2); }
  if (dot(cross(a0, a1), a2) < 0.f) a2 = -a2;
  SVD out;
  out.V = {{a0, a1, a2}};
  V3 u0, u1;
  const float eps = 1e-8f;
  if (sig.x > eps) u0 = normalizeFast(mul(F, a0));
  else u0 = v3(1.f, 0.f, 0.f);
  if (sig.y > eps) {
    const V3 Fv1 = mul(F, a1);
    u1 = Fv1 - dot(Fv1, u0) * u0;
    const float l2 = dot(u1, u1);
    if (l2 > eps * eps) u1 = u1 * rsqrtf(l2);
    else u1 = normalizeFast(cross(v3(0.f, 1.f, 0.f), u0) + splat(1e-4f));
  } else {
    V3 a = cross(u0, v3(0.f, 1.f, 0.f));
    if (dot(a, a) < 1e-8f) a = cross(u0, v3(1.f, 0.f, 0.f));
    u1 = normalizeFast(a);
  }
  const V3 u2 = cross(u0, u1);
  if (det(F) < 0.f) sig.z = -sig.z;
  out.U = {{u0, u1, u2}};
  out.sig = sig;
  return out;
}

// U diag(d) V^T (common.js:182-184)
__device__ __forceinline__ M3 diagMul(const M3& U, V3 d, const M3& V) {
  M3 Ud = {{U.c[0] * d.x, U.c[1] * d.y, U.c[2] * d.z}};
  return mul(Ud, transpose(V));
}

// ----------------------------------------------------------------- StVK-Hencky
// common.js:186-201
__device__ __forceinline__ V3 safeSig(V3 s) { return vclamp(s, 1e-3f, 1e3f); }
__device__ __forceinline__ float stvkPsi(V3 sig, float mu, float lam) {
  V3 e = vlog(safeSig(sig));
  float tr = e.x + e.y + e.z;
  return mu * dot(e, e) + 0.5f * lam * tr * tr;
}
__device__ __forceinline__ V3 stvkDPsi(V3 sig, float mu, float lam) {
  V3 s = safeSig(sig);
  V3 e = vlog(s);
  float tr = e.x + e.y + e.z;
  return (2.f * mu * e + splat(lam * tr)) / s;
}

// ----------------------------------------------------------------- return maps
// Drucker-Prager (common.js:205-221)
__device__ __forceinline__ V3 rmDruckerPrager(V3 sig, const MatDev& m) {
  float alpha = m.p0, coh = m.p1;
  V3 e = vlog(safeSig(sig)) - splat(coh);
  float tr = e.x + e.y + e.z;
  V3 dev = e - splat(tr / 3.f);
  float dn = length(dev);
  if (dn < 1e-9f || tr > 0.f) return vexp(splat(coh));
  float dg = dn + alpha * (3.f * m.lam + 2.f * m.mu) / (2.f * m.mu) * tr;
  if (dg <= 0.f) return sig;
  V3 en = e - (dg / dn) * dev;
  return vexp(en + splat(coh));
}
// Von Mises (common.js:223-234)
__device__ __forceinline__ V3 rmVonMises(V3 sig, const MatDev& m) {
  float sigY = m.p0;
  V3 e = vlog(safeSig(sig));
  float tr = e.x + e.y + e.z;
  V3 dev = e - splat(tr / 3.f);
  float dn = length(dev);
  float dg = dn - sigY / (2.f * m.mu);
  if (dg <= 0.f || dn < 1e-9f) return sig;
  V3 en = e - (dg / dn) * dev;
  return vexp(en);
}
// Herschel-Bulkley, b-bar-e form with bisection (common.js:236-280)
__device__ __forceinline__ V3 rmHerschelBulkley(V3 sig, const MatDev& m, float dt) {
  float sigY = m.p0, hexp = m.p1, eta = m.p2;
  V3 s3 = safeSig(sig);
  float J = s3.x * s3.y * s3.z;
  V3 bbar = s3 * s3 * powf(J, (float)(-2.0 / 3.0));
  float trb = bbar.x + bbar.y + bbar.z;
  V3 devb = bbar - splat(trb / 3.f);
  float sPre = m.mu * length(devb);
  float sY = (float)0.816496580927726 * sigY;  // sqrt(2/3)
  if (sPre <= sY || sPre < 1e-12f) return sig;
  float muT = (trb / 3.f) * m.mu;
  float sNew;
  if (fabsf(hexp - 1.f) < 1e-3f || eta < 1e-9f) {
    sNew = sPre - (sPre - sY) / (1.f + eta / (2.f * muT * dt));
  } else {
    float ih = 1.f / hexp;
    float ei = powf(eta, ih);
    float lo = sY, hi = sPre;
#pragma unroll 1
    for (int it = 0; it < 18; ++it) {
      float mid = 0.5f * (lo + hi);
      float g = ei * (mid - sPre) + 2.f * muT * dt * powf(fmaxf(mid - sY, 0.f), ih);
      if (g > 0.f) hi = mid;
      else lo = mid;
    }
    sNew = 0.5f * (lo + hi);
  }
  V3 bNew = devb * (sNew / sPre) + splat(trb / 3.f);
  bNew = vmaxs(bNew, 1e-6f);
  float detB = bNew.x * bNew.y * bNew.z;
  bNew = bNew * powf(detB, (float)(-1.0 / 3.0));
  return vsqrt(bNew) * powf(J, (float)(1.0 / 3.0));
}
// NACC, b^E form with fracture-friendly hardening (common.js:287-364)
__device__ __forceinline__ V3 rmNACC(V3 sig, const MatDev& m, float alphaIn, float& alphaOut) {
  float beta = m.p1, xi = m.p2, Mf = m.p3, mu = m.mu;
  float kappa = (float)(2.0 / 3.0) * mu + m.lam;
  float alpha = alphaIn;
  V3 s3 = safeSig(sig);
  float Jtr = s3.x * s3.y * s3.z;
  V3 b2 = s3 * s3;
  float trb = b2.x + b2.y + b2.z;
  V3 devb = b2 - splat(trb / 3.f);
  V3 sHat = mu * powf(Jtr, (float)(-2.0 / 3.0)) * devb;
  float sNorm = length(sHat);
  const float sqrt15 = (float)1.224744871391589;  // sqrt(1.5)
  float q = sqrt15 * sNorm;
  float p = -0.5f * kappa * (Jtr * Jtr - 1.f);
  alpha = clampf(alpha, -0.25f, 0.4f);
  float p0 = kappa * (0.00001f + sinhf(fminf(xi * fmaxf(-alpha, 0.f), 4.f)));
  float b = 1.f + 2.f * beta;
  V3 outSig = sig;
  if (p > p0) {
    float Jn = sqrtf(fmaxf(-2.f * p0 / kappa + 1.f, 1e-6f));
    outSig = splat(powf(Jn, (float)(1.0 / 3.0)));
    alpha = alpha + logf(Jtr / Jn);
  } else if (p < -beta * p0) {
    float Jn = sqrtf(fmaxf(2.f * beta * p0 / kappa + 1.f, 1e-6f));
    outSig = splat(powf(Jn, (float)(1.0 / 3.0)));
    alpha = alpha + logf(Jtr / Jn);
  } else {
    float y = b * q * q + Mf * Mf * (p + beta * p0) * (p - p0);
    if (y > 1e-4f && sNorm > 1e-9f) {
      if (p0 > 1e-4f && p < p0 - 1e-4f && p > -beta * p0 + 1e-4f) {
        float pc = (1.f - beta) * p0 * 0.5f;
        float lenDir = sqrtf((pc - p) * (pc - p) + (-q) * (-q));
        if (lenDir > 1e-9f) {
          float Dp = (pc - p) / lenDir;
          float Dq = -q / lenDir;
          float Aq = Mf * Mf * Dp * Dp + b * Dq * Dq;
          float Bq = Mf * Mf * Dp * (2.f * pc - p0 + beta * p0);
          float Cq = Mf * Mf * (pc + beta * p0) * (pc - p0);
          float disc = Bq * Bq - 4.f * Aq * Cq;
          if (disc > 0.f && fabsf(Aq) > 1e-12f) {
            float l1 = (-Bq + sqrtf(disc)) / (2.f * Aq);
            float l2 = (-Bq - sqrtf(disc)) / (2.f * Aq);
            float px1 = pc + l1 * Dp;
            float px2 = pc + l2 * Dp;
            float px = px1;
            if ((p - pc) * (px2 - pc) > 0.f) px = px2;
            float Jx2 = -2.f * px / kappa + 1.f;
            if (Jx2 > 1e-8f) {
              float Jx = sqrtf(Jx2);
              if (Jx > 1e-4f) alpha = alpha + logf(Jtr / Jx);
            }
          }
        }
      }
      float qN = Mf * sqrtf(fmaxf(-(p + beta * p0) * (p - p0), 0.f) / b);
      float sNewNorm = qN / sqrt15;
      V3 bNew = (powf(Jtr, (float)(2.0 / 3.0)) / mu) * (sNewNorm / sNorm) * sHat + splat(trb / 3.f);
      bNew = vmaxs(bNew, 1e-6f);
      outSig = vsqrt(bNew);
    }
  }
  alphaOut = alpha;
  return outSig;
}
// Snow hardening of mu, lambda (common.js:366-375)
__device__ __forceinline__ MatDev hardenedMat(const MatDev& m, float state) {
  MatDev mm = m;
  if (m.kind == kKindSnow) {
    float s = expf(fminf(m.p2 * (1.f - state), 5.f));
    mm.mu = m.mu * s;
    mm.lam = m.lam * s;
  }
  return mm;
}
// Dispatch on the material kind (common.js:377-396)
__device__ __forceinline__ V3 returnMap(V3 sig, const MatDev& m, float state, float dt, float& stateOut) {
  stateOut = state;
  switch (m.kind) {
    case 1u: return rmDruckerPrager(sig, m);
    case 2u: return rmNACC(sig, m, state, stateOut);
    case 3u: return rmVonMises(sig, m);
    case 4u: return rmHerschelBulkley(sig, m, dt);
    case 5u: {
      V3 sNew = v3(clampf(sig.x, 1.f - m.p0, 1.f + m.p1), clampf(sig.y, 1.f - m.p0, 1.f + m.p1),
                   clampf(sig.z, 1.f - m.p0, 1.f + m.p1));
      float jOld = sig.x * sig.y * sig.z;
      float jNew = sNew.x * sNew.y * sNew.z;
      stateOut = clampf(state * jOld / fmaxf(jNew, 1e-6f), 0.2f, 2.f);
      return sNew;
    }
    default: return sig;
  }
}

}  // namespace xpbi
