// Neighbour-gather kernels of the XPBI substep, one thread per particle slot
// in cell order. Each restates one compute entry point of
// web/js/shaders/simkernels.js (cited per kernel) with the same stencil walk
// (dz outer, dy inner, candidates ascending over the row-merged range of
// three x-adjacent cells, capped at 384) and the same f32 operation order.
//
// Batched handles: every slot belongs to one scene (sceneOf); its grid, cell
// table range, uniforms and material table come from that scene, and a
// neighbour stencil never leaves the scene's own cells. Passes beyond a
// scene's iteration budget copy velIn to velOut so the shared ping-pong
// parity stays consistent for every scene.
#include "xpbi_math.cuh"

namespace xpbi {

namespace {

constexpr int kThreads = 128;

struct Ctx {
  const SceneDev* __restrict__ scene;
  const MatDev* __restrict__ mats;   // this scene's 8 materials
};

__device__ __forceinline__ Ctx ctxOf(const Bufs& b, uint32_t i) {
  uint32_t s = b.S > 1 ? (uint32_t)b.sceneOf[i] : 0u;
  const SceneDev* S = b.scenes + s;
  return Ctx{S, b.mats + S->matBase};
}

// material index stored as a float value in pos.w (simkernels.js:41-44)
__device__ __forceinline__ uint32_t matOfW(float w) {
  if (!(w > 0.f)) return 0u;
  uint32_t m = (uint32_t)w;
  return m > 7u ? 7u : m;
}
__device__ __forceinline__ bool isSolid(const MatDev* mats, uint32_t mi) { return mats[mi].kind != kKindWater; }

// Stencil walk over the 9 row-merged ranges (simkernels.js:62-74).
template <class Body>
__device__ __forceinline__ void forStencil(const SceneDev& S, const uint32_t* __restrict__ cellStart, V3 x,
                                           Body&& body) {
  I3 cc = cellCoord(S, x);
  const int x0 = max(cc.x - 1, 0);
  const int x1 = min(cc.x + 1, S.dims[0] - 1);
#pragma unroll 1
  for (int dz = -1; dz <= 1; ++dz) {
    const int z = cc.z + dz;
    if (z < 0 || z >= S.dims[2]) continue;
#pragma unroll 1
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = cc.y + dy;
      if (y < 0 || y >= S.dims[1]) continue;
      const uint32_t c0 = S.cellBase + cellIndex(S, x0, y, z);
      const uint32_t c2 = S.cellBase + cellIndex(S, x1, y, z);
      const uint32_t beg = cellStart[c0];
      const uint32_t end = min(cellStart[c2 + 1], beg + kRowCap);
#pragma unroll 1
      for (uint32_t bb = beg; bb < end; ++bb) body(bb);
    }
  }
}

// velocityGradient (simkernels.js:224-245)
__device__ __forceinline__ M3 velocityGradient(const Bufs& b, const Ctx& cx, uint32_t i, V3 xi, V3 vi,
                                               const float4* __restrict__ velIn) {
  const SceneDev& S = *cx.scene;
  const M3 Li = loadM(b.L, b.N, i);
  M3 G = mzero();
  forStencil(S, b.cellStart, xi, [&](uint32_t j) {
    if (j == i) return;
    const float4 pj = b.posS[j];
    if (!isSolid(cx.mats, matOfW(pj.w))) return;
    V3 dxv = xi - xyz(pj);
    if (dot(dxv, dxv) < S.support2) {
      V3 gt = mul(Li, kernelGradW(S, dxv));
      float4 vb = velIn[j];
      V3 dv = (xyz(vb) - vi) * vb.w;
      G = madd(G, M3{{dv * gt.x, dv * gt.y, dv * gt.z}});
    }
  });
  return G;
}

// ---------------------------------------------------------------- computeL
// simkernels.js:189-221
__global__ void __launch_bounds__(kThreads) k_computeL(Bufs b) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  const float4* __restrict__ velIn = b.velS[0];
  V3 xi = xyz(b.posS[i]);
  M3 A = mzero();
  forStencil(S, b.cellStart, xi, [&](uint32_t j) {
    if (j == i) return;
    V3 pb = xyz(b.posS[j]);
    V3 dxv = xi - pb;
    if (dot(dxv, dxv) < S.support2) {
      V3 g = kernelGradW(S, dxv);
      V3 r = pb - xi;
      M3 o = {{g * r.x, g * r.y, g * r.z}};
      A = madd(A, mscale(o, velIn[j].w));
    }
  });
  SVD s = svd3(A);
  const float tol = 0.2f;
  V3 inv = splat(0.f);
  if (fabsf(s.sig.x) > tol) inv.x = 1.f / s.sig.x;
  if (fabsf(s.sig.y) > tol) inv.y = 1.f / s.sig.y;
  if (fabsf(s.sig.z) > tol) inv.z = 1.f / s.sig.z;
  storeM(b.L, b.N, i, diagMul(s.V, inv, s.U));
}

__device__ __forceinline__ void storeSp(float4* __restrict__ Sp, uint32_t i, const M3& m, V3 s) {
  Sp[3 * (size_t)i] = make_float4(m.c[0].x, m.c[0].y, m.c[0].z, s.x);
  Sp[3 * (size_t)i + 1] = make_float4(m.c[1].x, m.c[1].y, m.c[1].z, s.y);
  Sp[3 * (size_t)i + 2] = make_float4(m.c[2].x, m.c[2].y, m.c[2].z, s.z);
}

// ---------------------------------------------------------------- solveA
// Inelastic constraint pass A (simkernels.js:248-309)
__global__ void __launch_bounds__(kThreads) k_solveA(Bufs b, int k, const float4* __restrict__ velIn) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  if (k >= S.iterations) return;
  const float4 pi = b.posS[i];
  const uint32_t mi = matOfW(pi.w);
  if (!isSolid(cx.mats, mi)) return;  // water: Sp is never read
  const float st = b.stateS[i];
  MatDev m = hardenedMat(cx.mats[mi], st);
  const V3 xi = xyz(pi);
  const float4 vi4 = velIn[i];
  const V3 vi = xyz(vi4);
  const M3 Fn = loadM(b.FS, b.N, i);
  const M3 gradV = velocityGradient(b, cx, i, xi, vi, velIn);
  const M3 Ftr = mul(madd(mident(), mscale(gradV, S.dt)), Fn);
  const SVD sv = svd3(Ftr);
  float stOut;
  const V3 sig = returnMap(sv.sig, m, st, S.dt, stOut);
  const float psi = stvkPsi(sig, m.mu, m.lam);
  const float C = sqrtf(fmaxf(2.f * psi, 0.f));
  if (C < 1e-7f) {
    storeSp(b.Sp, i, mzero(), splat(0.f));
    return;
  }
  const V3 dpsi = stvkDPsi(sig, m.mu, m.lam);
  const M3 Pk = diagMul(sv.U, dpsi / C, sv.V);
  const M3 GL = mul(mul(Pk, transpose(Fn)), loadM(b.L, b.N, i));
  float denom = 0.f, cdot = 0.f;
  V3 sgrad = splat(0.f);
  forStencil(S, b.cellStart, xi, [&](uint32_t j) {
    if (j == i) return;
    const float4 pj = b.posS[j];
    const uint32_t mj = matOfW(pj.w);
    if (!isSolid(cx.mats, mj)) return;
    V3 dxv = xi - xyz(pj);
    if (dot(dxv, dxv) < S.support2) {
      float4 vb = velIn[j];
      V3 gb = vb.w * mul(GL, kernelGradW(S, dxv));
      denom = denom + dot(gb, gb) / cx.mats[mj].mass;
      sgrad = sgrad - gb;
      cdot = cdot + dot(gb, xyz(vb));
    }
  });
  denom = denom + dot(sgrad, sgrad) / m.mass;
  cdot = cdot + dot(sgrad, vi);
  const float g = S.kDamp;
  const float lam0 = b.lam[i];
  const float dlam = S.omega * (-C - S.alphaT * lam0 - g * S.dt * cdot) / ((1.f + g) * denom + S.alphaT);
  b.lam[i] = lam0 + dlam;
  storeSp(b.Sp, i, mscale(GL, dlam), sgrad * dlam);
}

// applyBoundary (simkernels.js:369-404)
__device__ __forceinline__ V3 applyBoundary(const SceneDev& S, V3 xcIn, V3 vIn, V3 xn, float fric) {
  V3 vv = vIn, xq = xcIn;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float lo = S.dmin[k], hi = S.dmax[k];
    if (xq[k] < lo || xq[k] > hi) {
      const float bound = xq[k] < lo ? lo : hi;
      const float vnNew = (bound - xn[k]) / S.dt;
      const float dvn = fabsf(vnNew - vv[k]);
      V3 vt = vv;
      vt[k] = 0.f;
      const float vtl = length(vt);
      if (vtl > 1e-9f) {
        const float drop = fminf(fric * dvn, vtl);
        vv = vv - vt / vtl * drop;
      }
      vv[k] = vnNew;
      xq = xn + S.dt * vv;
    }
  }
  if (S.colActive > 0.5f) {
    const V3 cp = v3(S.colPos[0], S.colPos[1], S.colPos[2]);
    const V3 cv = v3(S.colVel[0], S.colVel[1], S.colVel[2]);
    const V3 d = xq - cp;
    const float dist = length(d);
    if (dist < S.colR && dist > 1e-9f) {
      const V3 n = d / dist;
      const float vOut = dot(vv - cv, n);
      const float vGoal = fminf((S.colR - dist) / S.dt, 0.6f);
      if (vOut < vGoal) vv = vv + n * (vGoal - vOut);
    }
  }
  return vv;
}

// ---------------------------------------------------------------- solveB
// Constraint dv gather + contact correction + boundaries (simkernels.js:315-366)
__global__ void __launch_bounds__(kThreads) k_solveB(Bufs b, int k, const float4* __restrict__ velIn,
                                                      float4* __restrict__ velOut) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  const float4 vi4 = velIn[i];
  if (k >= S.iterations) {
    velOut[i] = vi4;
    return;
  }
  const float4 pi = b.posS[i];
  const uint32_t mi = matOfW(pi.w);
  const MatDev& m = cx.mats[mi];
  const V3 xi = xyz(pi);
  V3 dv = splat(0.f), corr = splat(0.f);
  if (m.kind != kKindWater) {
    const float4 s0 = b.Sp[3 * (size_t)i], s1 = b.Sp[3 * (size_t)i + 1], s2 = b.Sp[3 * (size_t)i + 2];
    dv = v3(s0.w, s1.w, s2.w);
    const float Vi = vi4.w;
    const V3 xci = xi + S.dt * xyz(vi4);
    const float minD = S.minD;
    const float massI = m.mass;
    forStencil(S, b.cellStart, xi, [&](uint32_t j) {
      if (j == i) return;
      const float4 pj = b.posS[j];
      const uint32_t mj = matOfW(pj.w);
      if (!isSolid(cx.mats, mj)) return;
      const V3 pb = xyz(pj);
      const V3 dxp = pb - xi;
      if (dot(dxp, dxp) < S.support2) {
        const float4 a0 = b.Sp[3 * (size_t)j], a1 = b.Sp[3 * (size_t)j + 1], a2 = b.Sp[3 * (size_t)j + 2];
        const M3 Sb = {{xyz(a0), xyz(a1), xyz(a2)}};
        dv = dv + Vi * mul(Sb, kernelGradW(S, dxp));
        const V3 xcb = pb + S.dt * xyz(velIn[j]);
        const V3 dxc = xci - xcb;
        const float dist = length(dxc);
        if (dist < minD && dist > 1e-9f) {
          const float mb = cx.mats[mj].mass;
          const float w = mb / (massI + mb);
          corr = corr + dxc / dist * ((minD - dist) * w);
        }
      }
    });
  }
  V3 dvv = dv / (m.mass * S.dt);
  const float dvl = length(dvv);
  if (dvl > S.dvCap) dvv = dvv * (S.dvCap / dvl);
  V3 v = xyz(vi4) + dvv + corr * (S.contactOmega / S.dt);
  v = applyBoundary(S, xi + S.dt * v, v, xi, m.boundFriction);
  velOut[i] = make_float4(v.x, v.y, v.z, vi4.w);
}

__device__ __forceinline__ bool pbfActive(const SceneDev& S, int k) {
  return S.hasWater && k < S.iterations && (S.pbfIterations < 0 || k < S.pbfIterations);
}

// ---------------------------------------------------------------- pbfA
// PBF density multiplier (simkernels.js:407-439)
__global__ void __launch_bounds__(kThreads) k_pbfA(Bufs b, int k, const float4* __restrict__ velIn) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  if (!pbfActive(S, k)) return;
  const float4 pi = b.posS[i];
  const uint32_t mi = matOfW(pi.w);
  if (isSolid(cx.mats, mi)) {
    b.pbfLam[i] = 0.f;
    return;
  }
  const MatDev& m = cx.mats[mi];
  const float rho0 = m.density;
  const V3 xn = xyz(pi);
  const V3 xci = xn + S.dt * xyz(velIn[i]);
  float rho = m.mass * S.w00;
  V3 gradSum = splat(0.f);
  float grad2 = 0.f;
  forStencil(S, b.cellStart, xn, [&](uint32_t j) {
    if (j == i) return;
    const float4 pj = b.posS[j];
    const V3 xcb = xyz(pj) + S.dt * xyz(velIn[j]);
    const V3 dxv = xci - xcb;
    if (dot(dxv, dxv) < S.support2) {
      const float mb = cx.mats[matOfW(pj.w)].mass;
      rho = rho + mb * kernelPoly6(S, length(dxv));
      const V3 g = kernelSpikyGrad(S, dxv) * (mb / rho0);
      gradSum = gradSum + g;
      grad2 = grad2 + dot(g, g);
    }
  });
  const float C = fmaxf(rho / rho0 - 1.f, 0.f);
  b.pbfLam[i] = -C / (grad2 + dot(gradSum, gradSum) + S.pbfEps);
}

// ---------------------------------------------------------------- pbfB
// PBF position correction with s_corr (simkernels.js:441-477)
__global__ void __launch_bounds__(kThreads) k_pbfB(Bufs b, int k, const float4* __restrict__ velIn,
                                                    float4* __restrict__ velOut) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  const float4 vi4 = velIn[i];
  if (!pbfActive(S, k)) {
    velOut[i] = vi4;
    return;
  }
  const float4 pi = b.posS[i];
  const uint32_t mi = matOfW(pi.w);
  const V3 xn = xyz(pi);
  const V3 xci = xn + S.dt * xyz(vi4);
  V3 dp = splat(0.f);
  const float li = b.pbfLam[i];
  const bool iAmWater = !isSolid(cx.mats, mi);
  const float w0 = fmaxf(S.w0, 1e-12f);
  forStencil(S, b.cellStart, xn, [&](uint32_t j) {
    if (j == i) return;
    const float4 pj = b.posS[j];
    const uint32_t mj = matOfW(pj.w);
    const bool bWater = !isSolid(cx.mats, mj);
    if (!(iAmWater || bWater)) return;
    const V3 xcb = xyz(pj) + S.dt * xyz(velIn[j]);
    const V3 dxv = xci - xcb;
    if (dot(dxv, dxv) < S.support2) {
      const MatDev& mw = cx.mats[bWater ? mj : mi];
      const float lb = b.pbfLam[j];
      const float w = kernelPoly6(S, length(dxv));
      const float sCorr = -S.sCorrK * powf(w / w0, 4.f);
      dp = dp + (li + lb + sCorr) * kernelSpikyGrad(S, dxv) * (mw.mass / mw.density);
    }
  });
  const float scale = iAmWater ? 1.f : 0.5f;
  const V3 v = xyz(vi4) + dp * (scale / S.dt);
  velOut[i] = make_float4(v.x, v.y, v.z, vi4.w);
}

// ---------------------------------------------------------------- xsph
// simkernels.js:480-507
__global__ void __launch_bounds__(kThreads) k_xsph(Bufs b, const float4* __restrict__ velIn,
                                                    float4* __restrict__ velOut) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  const float4 pi = b.posS[i];
  const V3 xi = xyz(pi);
  const float4 vi4 = velIn[i];
  const V3 vi = xyz(vi4);
  const bool iSolid = isSolid(cx.mats, matOfW(pi.w));
  V3 acc = splat(0.f);
  forStencil(S, b.cellStart, xi, [&](uint32_t j) {
    if (j == i) return;
    const float4 pj = b.posS[j];
    if (isSolid(cx.mats, matOfW(pj.w)) != iSolid) return;
    const V3 dxv = xi - xyz(pj);
    if (dot(dxv, dxv) < S.support2) {
      const float4 vb = velIn[j];
      acc = acc + vb.w * (xyz(vb) - vi) * kernelW(S, length(dxv));
    }
  });
  float c = S.xsphC;
  if (!iSolid) c = S.xsphC * 10.f;
  const V3 v = vi + c * acc;
  velOut[i] = make_float4(v.x, v.y, v.z, vi4.w);
}

// ---------------------------------------------------------------- updateF + integrate
// Final F with return mapping (simkernels.js:510-525) fused with the CFL
// clamp and position update (simkernels.js:528-542). Outputs go to the
// "current" arrays, so neighbours still read the unclamped sorted inputs.
__global__ void __launch_bounds__(kThreads) k_updateF_integrate(Bufs b, const float4* __restrict__ velIn) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  const float4 pi = b.posS[i];
  const uint32_t mi = matOfW(pi.w);
  const float4 vi4 = velIn[i];
  const float st = b.stateS[i];
  M3 Fn = loadM(b.FS, b.N, i);
  float stOut = st;
  if (isSolid(cx.mats, mi)) {
    MatDev m = hardenedMat(cx.mats[mi], st);
    const M3 gradV = velocityGradient(b, cx, i, xyz(pi), xyz(vi4), velIn);
    const M3 Ftr = mul(madd(mident(), mscale(gradV, S.dt)), Fn);
    const SVD sv = svd3(Ftr);
    const V3 sig = returnMap(sv.sig, m, st, S.dt, stOut);
    Fn = diagMul(sv.U, safeSig(sig), sv.V);
  }
  storeM(b.F, b.N, i, Fn);
  b.state[i] = stOut;
  V3 v = xyz(vi4);
  const float vl = length(v);
  if (vl > S.vmaxCFL) v = v * (S.vmaxCFL / vl);
  b.vel[i] = make_float4(v.x, v.y, v.z, vi4.w);
  V3 x = xyz(pi) + S.dt * v;
  x = v3(clampf(x.x, S.dmin[0], S.dmax[0]), clampf(x.y, S.dmin[1], S.dmax[1]), clampf(x.z, S.dmin[2], S.dmax[2]));
  b.pos[i] = make_float4(x.x, x.y, x.z, pi.w);
}

inline unsigned grid(uint32_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

}  // namespace

void launch_computeL(const Bufs& b, cudaStream_t st) { k_computeL<<<grid(b.N), kThreads, 0, st>>>(b); }
void launch_solveA(const Bufs& b, int k, const float4* velIn, cudaStream_t st) {
  k_solveA<<<grid(b.N), kThreads, 0, st>>>(b, k, velIn);
}
void launch_solveB(const Bufs& b, int k, const float4* velIn, float4* velOut, cudaStream_t st) {
  k_solveB<<<grid(b.N), kThreads, 0, st>>>(b, k, velIn, velOut);
}
void launch_pbfA(const Bufs& b, int k, const float4* velIn, cudaStream_t st) {
  k_pbfA<<<grid(b.N), kThreads, 0, st>>>(b, k, velIn);
}
void launch_pbfB(const Bufs& b, int k, const float4* velIn, float4* velOut, cudaStream_t st) {
  k_pbfB<<<grid(b.N), kThreads, 0, st>>>(b, k, velIn, velOut);
}
void launch_xsph(const Bufs& b, const float4* velIn, float4* velOut, cudaStream_t st) {
  k_xsph<<<grid(b.N), kThreads, 0, st>>>(b, velIn, velOut);
}
void launch_updateF_integrate(const Bufs& b, const float4* velIn, cudaStream_t st) {
  k_updateF_integrate<<<grid(b.N), kThreads, 0, st>>>(b, velIn);
}

}  // namespace xpbi
