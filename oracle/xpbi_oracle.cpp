// XPBI substep CPU oracle — TEST INFRASTRUCTURE ONLY.
//
// This file is the checker for the CUDA library, never part of it: only the
// tests, the smoke check and the CPU-baseline leg of the benchmark load it.
// It restates, dispatch by dispatch, the reference WebGPU substep of
// Chiplis/xpbi-webgpu:
//   web/js/sim.js:220-272            encodeSubstep (dispatch order, ping-pong)
//   web/js/shaders/simkernels.js     every compute entry point (cited per function)
//   web/js/shaders/common.js         SPH kernels, svd3, StVK-Hencky, return maps
// Each "dispatch" runs its invocations in ascending index order. That fixes the
// otherwise unordered atomics: in `scatter` the lowest particle index of a cell
// takes the highest slot, so each cell lists its particles by descending
// previous index. Everything else is invocation-independent, so the
// OpenMP-parallel loops give bit-identical results for any thread count.
//
// Parity status: pinned against the reference's own kernels. Its WGSL cannot
// execute on a WebGPU adapter here, so oracle/wgsl_ref.py translates that
// WGSL mechanically into C++ and runs it in sim.js's dispatch order; the f32
// instantiation below equals it bit for bit (sort, state, multipliers) on
// every reference demo scene and benchmark config, fresh and developed
// (tests/test_oracle_vs_reference.py). WGSL leaves determinant()'s
// evaluation order to the implementation: both use the triple product
// c0 . (c1 x c2). The Drucker-Prager return map and the StVK-Hencky energy
// are also checked against the reference's NumPy prototype
// (prototype/xpbi2d.py:93-116) through committed fixtures.
//
// Two instantiations: float (WGSL f32 semantics, the parity oracle) and double
// (the FP64 error reference of the same substep). Cell coordinates are always
// computed in f32 so both share one neighbourhood structure.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr uint32_t MAT_SNOW = 5u, MAT_WATER = 6u;
constexpr uint32_t ROW_CAP = 384u;  // simkernels.js:73

template <class R> struct V3 {
  R x, y, z;
  R& operator[](int k) { return k == 0 ? x : (k == 1 ? y : z); }
  R operator[](int k) const { return k == 0 ? x : (k == 1 ? y : z); }
};
template <class R> V3<R> v3(R a, R b, R c) { return V3<R>{a, b, c}; }
template <class R> V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> V3<R> operator/(V3<R> a, V3<R> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class R> V3<R> splat(R s) { return {s, s, s}; }
template <class R> R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> R length(V3<R> a) { return std::sqrt(dot(a, a)); }
template <class R> V3<R> normalize(V3<R> a) { return a / length(a); }
template <class R> V3<R> cross(V3<R> a, V3<R> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> R fmin_(R a, R b) { return std::fmin(a, b); }
template <class R> R fmax_(R a, R b) { return std::fmax(a, b); }
template <class R> R clampf(R v, R lo, R hi) { return fmin_(fmax_(v, lo), hi); }
template <class R> V3<R> vclamp(V3<R> v, V3<R> lo, V3<R> hi) {
  return {clampf(v.x, lo.x, hi.x), clampf(v.y, lo.y, hi.y), clampf(v.z, lo.z, hi.z)};
}
template <class R> V3<R> vmax(V3<R> v, V3<R> m) { return {fmax_(v.x, m.x), fmax_(v.y, m.y), fmax_(v.z, m.z)}; }
template <class R> V3<R> vlog(V3<R> v) { return {std::log(v.x), std::log(v.y), std::log(v.z)}; }
template <class R> V3<R> vexp(V3<R> v) { return {std::exp(v.x), std::exp(v.y), std::exp(v.z)}; }
template <class R> V3<R> vsqrt(V3<R> v) { return {std::sqrt(v.x), std::sqrt(v.y), std::sqrt(v.z)}; }

// Column-major 3x3 (WGSL mat3x3f): c[j] is column j.
template <class R> struct M3 { V3<R> c[3]; };
template <class R> M3<R> mzero() { return {{splat<R>(0), splat<R>(0), splat<R>(0)}}; }
template <class R> M3<R> mident() { return {{v3<R>(1, 0, 0), v3<R>(0, 1, 0), v3<R>(0, 0, 1)}}; }
template <class R> V3<R> mul(const M3<R>& A, V3<R> v) { return A.c[0] * v.x + A.c[1] * v.y + A.c[2] * v.z; }
template <class R> M3<R> mul(const M3<R>& A, const M3<R>& B) {
  return {{mul(A, B.c[0]), mul(A, B.c[1]), mul(A, B.c[2])}};
}
template <class R> M3<R> transpose(const M3<R>& A) {
  return {{v3(A.c[0].x, A.c[1].x, A.c[2].x), v3(A.c[0].y, A.c[1].y, A.c[2].y),
           v3(A.c[0].z, A.c[1].z, A.c[2].z)}};
}
template <class R> M3<R> madd(const M3<R>& A, const M3<R>& B) {
  return {{A.c[0] + B.c[0], A.c[1] + B.c[1], A.c[2] + B.c[2]}};
}
template <class R> M3<R> mscale(const M3<R>& A, R s) { return {{A.c[0] * s, A.c[1] * s, A.c[2] * s}}; }
template <class R> R det(const M3<R>& A) { return dot(A.c[0], cross(A.c[1], A.c[2])); }

// ---------------------------------------------------------------- params
// Decodes the reference's 256-byte Params uniform (sim.js:159-186,
// common.js:35-60) and the 8 x 16-word Material table (sim.js:84-99,
// common.js:21-33).
struct Mat {
  double mu, lam, density;
  uint32_t kind;
  double p0, p1, p2, p3, boundFriction, mass;
};
template <class R> struct MatR {
  R mu, lam, density;
  uint32_t kind;
  R p0, p1, p2, p3, boundFriction, mass;
};

template <class R> struct Params {
  float originF[3], cellF;  // f32 copies: cell coordinates are always f32
  int dims[3];
  uint32_t numCells, N;
  R domainMin[3], domainMax[3], dt, h, support, gravity[3];
  R colliderPos[3], colliderR, colliderVel[3], colliderActive;
  R V0, xsphC, omega, pbfEps, sCorrK, contactOmega, kDamp;
  MatR<R> mats[8];
};

template <class R> Params<R> decode(const uint32_t* w, const uint32_t* m) {
  auto f = [&](int k) { float x; std::memcpy(&x, &w[k], 4); return x; };
  Params<R> p{};
  for (int k = 0; k < 3; ++k) {
    p.originF[k] = f(k);
    p.dims[k] = (int32_t)w[4 + k];
    p.domainMin[k] = (R)f(8 + k);
    p.domainMax[k] = (R)f(12 + k);
    p.gravity[k] = (R)f(16 + k);
    p.colliderPos[k] = (R)f(20 + k);
    p.colliderVel[k] = (R)f(24 + k);
  }
  p.cellF = f(3);
  p.numCells = w[7];
  p.dt = (R)f(11);
  p.h = (R)f(15);
  p.support = (R)f(19);
  p.colliderR = (R)f(23);
  p.colliderActive = (R)f(27);
  p.N = w[28];
  p.V0 = (R)f(29);
  p.xsphC = (R)f(30);
  p.omega = (R)f(31);
  p.pbfEps = (R)f(32);
  p.sCorrK = (R)f(33);
  p.contactOmega = (R)f(35);
  p.kDamp = (R)f(36);
  for (int i = 0; i < 8; ++i) {
    const uint32_t* q = m + 16 * i;
    auto g = [&](int k) { float x; std::memcpy(&x, &q[k], 4); return (R)x; };
    MatR<R>& M = p.mats[i];
    M.mu = g(0); M.lam = g(1); M.density = g(2); M.kind = q[3];
    M.p0 = g(4); M.p1 = g(5); M.p2 = g(6); M.p3 = g(7);
    M.boundFriction = g(12); M.mass = g(13);
  }
  return p;
}

// ------------------------------------------------------- SPH kernels
// common.js:63-94. Constant sub-expressions fold the way WGSL's abstract
// floats do: 16*pi, 64*pi are formed in f64 and rounded once to R.
template <class R> R kernelW(const Params<R>& P, R r) {
  R q = r / P.h;
  if (q >= R(2)) return R(0);
  R t = R(1) - R(0.5) * q;
  R sig = R(21) / (R(16.0 * 3.14159265) * P.h * P.h * P.h);
  return sig * t * t * t * t * (R(2) * q + R(1));
}
template <class R> V3<R> kernelGradW(const Params<R>& P, V3<R> dxv) {
  R r = length(dxv);
  R q = r / P.h;
  if (q >= R(2) || r < R(1e-9)) return splat<R>(0);
  R t = R(1) - R(0.5) * q;
  R sig = R(21) / (R(16.0 * 3.14159265) * P.h * P.h * P.h);
  R dwdq = sig * (R(-5) * q) * t * t * t;
  return dxv * (dwdq / (P.h * r));
}
template <class R> R kernelPoly6(const Params<R>& P, R r) {
  R H = P.support;
  if (r >= H) return R(0);
  R x = H * H - r * r;
  return R(315) / (R(64.0 * 3.14159265) * std::pow(H, R(9))) * x * x * x;
}
template <class R> V3<R> kernelSpikyGrad(const Params<R>& P, V3<R> dxv) {
  R H = P.support;
  R r = length(dxv);
  if (r >= H || r < R(1e-9)) return splat<R>(0);
  R t = H - r;
  return dxv * (R(-45) / (R(3.14159265) * std::pow(H, R(6))) * t * t / r);
}

// ------------------------------------------------------- grid helpers
// common.js:97-103; always f32 (see header).
struct I3 { int x, y, z; };
template <class R> I3 cellCoord(const Params<R>& P, V3<R> p) {
  float q[3] = {((float)p.x - P.originF[0]) / P.cellF, ((float)p.y - P.originF[1]) / P.cellF,
                ((float)p.z - P.originF[2]) / P.cellF};
  int c[3];
  for (int k = 0; k < 3; ++k) {
    float fl = std::floor(q[k]);
    // saturating f32->i32 (NaN -> 0), then clamp to the grid
    fl = std::fmin(std::fmax(fl, 0.0f), (float)(P.dims[k] - 1));
    c[k] = (int)fl;
  }
  return {c[0], c[1], c[2]};
}
template <class R> uint32_t cellIndex(const Params<R>& P, I3 c) {
  return (uint32_t)c.x + (uint32_t)c.y * (uint32_t)P.dims[0] +
         (uint32_t)c.z * (uint32_t)(P.dims[0] * P.dims[1]);
}

// ------------------------------------------------------- svd3
// common.js:105-184: Jacobi eigen-decomposition of F^T F, 6 sweeps.
template <class R> void jacobiRot(M3<R>& S, M3<R>& V, int p, int q) {
  R Spq = S.c[q][p];
  R Spp = S.c[p][p];
  R Sqq = S.c[q][q];
  if (std::fabs(Spq) < R(1e-12)) return;
  R tau = (Sqq - Spp) / (R(2) * Spq);
  R t;
  if (tau >= R(0)) t = R(1) / (tau + std::sqrt(R(1) + tau * tau));
  else t = R(1) / (tau - std::sqrt(R(1) + tau * tau));
  R c = R(1) / std::sqrt(R(1) + t * t);
  R s = t * c;
  M3<R> Sn = S;
  for (int k = 0; k < 3; ++k) {
    R Skp = S.c[p][k], Skq = S.c[q][k];
    Sn.c[p][k] = c * Skp - s * Skq;
    Sn.c[q][k] = s * Skp + c * Skq;
  }
  M3<R> S2 = Sn;
  for (int k = 0; k < 3; ++k) {
    R Spk = Sn.c[k][p], Sqk = Sn.c[k][q];
    S2.c[k][p] = c * Spk - s * Sqk;
    S2.c[k][q] = s * Spk + c * Sqk;
  }
  S = S2;
  M3<R> Vn = V;
  for (int k = 0; k < 3; ++k) {
    R Vkp = V.c[p][k], Vkq = V.c[q][k];
    Vn.c[p][k] = c * Vkp - s * Vkq;
    Vn.c[q][k] = s * Vkp + c * Vkq;
  }
  V = Vn;
}

template <class R> struct SVD { M3<R> U; V3<R> sig; M3<R> V; };

template <class R> SVD<R> svd3(const M3<R>& F) {
  M3<R> S = mul(transpose(F), F);
  M3<R> V = mident<R>();
  for (int sweep = 0; sweep < 6; ++sweep) {
    jacobiRot(S, V, 0, 1);
    jacobiRot(S, V, 0, 2);
    jacobiRot(S, V, 1, 2);
  }
  V3<R> sig = v3(std::sqrt(fmax_(S.c[0][0], R(0))), std::sqrt(fmax_(S.c[1][1], R(0))),
                 std::sqrt(fmax_(S.c[2][2], R(0))));
  V3<R> a0 = V.c[0], a1 = V.c[1], a2 = V.c[2];
  if (sig.x < sig.y) { std::swap(sig.x, sig.y); std::swap(a0, a1); }
  if (sig.x < sig.z) { std::swap(sig.x, sig.z); std::swap(a0, a2); }
  if (sig.y < sig.z) { std::swap(sig.y, sig.z); std::swap(a1, a2); }
  if (dot(cross(a0, a1), a2) < R(0)) a2 = -a2;
  V = {{a0, a1, a2}};
  V3<R> u0, u1, u2;
  const R eps = R(1e-8);
  if (sig.x > eps) u0 = normalize(mul(F, a0));
  else u0 = v3<R>(1, 0, 0);
  if (sig.y > eps) {
    V3<R> Fv1 = mul(F, a1);
    u1 = Fv1 - dot(Fv1, u0) * u0;
    R l = length(u1);
    if (l > eps) u1 = u1 / l;
    else u1 = normalize(cross(v3<R>(0, 1, 0), u0) + splat<R>(R(1e-4)));
  } else {
    V3<R> a = cross(u0, v3<R>(0, 1, 0));
    if (length(a) < R(1e-4)) a = cross(u0, v3<R>(1, 0, 0));
    u1 = normalize(a);
  }
  u2 = cross(u0, u1);
  if (det(F) < R(0)) sig.z = -sig.z;
  return {{{u0, u1, u2}}, sig, V};
}

template <class R> M3<R> diagMul(const M3<R>& U, V3<R> d, const M3<R>& V) {
  M3<R> Ud = {{U.c[0] * d.x, U.c[1] * d.y, U.c[2] * d.z}};
  return mul(Ud, transpose(V));
}

// ------------------------------------------------------- StVK-Hencky
// common.js:186-201
template <class R> V3<R> safeSig(V3<R> s) { return vclamp(s, splat<R>(R(1e-3)), splat<R>(R(1e3))); }
template <class R> R stvkPsi(V3<R> sig, R mu, R lam) {
  V3<R> e = vlog(safeSig(sig));
  R tr = e.x + e.y + e.z;
  return mu * dot(e, e) + R(0.5) * lam * tr * tr;
}
template <class R> V3<R> stvkDPsi(V3<R> sig, R mu, R lam) {
  V3<R> s = safeSig(sig);
  V3<R> e = vlog(s);
  R tr = e.x + e.y + e.z;
  return (R(2) * mu * e + splat(lam * tr)) / s;
}

// ------------------------------------------------------- return maps
// Drucker-Prager, common.js:205-221
template <class R> V3<R> rmDruckerPrager(V3<R> sig, const MatR<R>& m) {
  R alpha = m.p0, coh = m.p1;
  V3<R> e = vlog(safeSig(sig)) - splat(coh);
  R tr = e.x + e.y + e.z;
  V3<R> dev = e - splat(tr / R(3));
  R dn = length(dev);
  if (dn < R(1e-9) || tr > R(0)) return vexp(splat(coh));
  R dg = dn + alpha * (R(3) * m.lam + R(2) * m.mu) / (R(2) * m.mu) * tr;
  if (dg <= R(0)) return sig;
  V3<R> en = e - (dg / dn) * dev;
  return vexp(en + splat(coh));
}
// Von Mises, common.js:223-234
template <class R> V3<R> rmVonMises(V3<R> sig, const MatR<R>& m) {
  R sigY = m.p0;
  V3<R> e = vlog(safeSig(sig));
  R tr = e.x + e.y + e.z;
  V3<R> dev = e - splat(tr / R(3));
  R dn = length(dev);
  R dg = dn - sigY / (R(2) * m.mu);
  if (dg <= R(0) || dn < R(1e-9)) return sig;
  V3<R> en = e - (dg / dn) * dev;
  return vexp(en);
}
// Herschel-Bulkley, common.js:236-280
template <class R> V3<R> rmHerschelBulkley(V3<R> sig, const MatR<R>& m, R dt) {
  R sigY = m.p0, hexp = m.p1, eta = m.p2;
  V3<R> s3 = safeSig(sig);
  R J = s3.x * s3.y * s3.z;
  V3<R> bbar = s3 * s3 * std::pow(J, R(-2.0 / 3.0));
  R trb = bbar.x + bbar.y + bbar.z;
  V3<R> devb = bbar - splat(trb / R(3));
  R sPre = m.mu * length(devb);
  R sY = R(std::sqrt(2.0 / 3.0)) * sigY;
  if (sPre <= sY || sPre < R(1e-12)) return sig;
  R muT = (trb / R(3)) * m.mu;
  R sNew;
  if (std::fabs(hexp - R(1)) < R(1e-3) || eta < R(1e-9)) {
    sNew = sPre - (sPre - sY) / (R(1) + eta / (R(2) * muT * dt));
  } else {
    R ih = R(1) / hexp;
    R ei = std::pow(eta, ih);
    R lo = sY, hi = sPre;
    for (int it = 0; it < 18; ++it) {
      R mid = R(0.5) * (lo + hi);
      R g = ei * (mid - sPre) + R(2) * muT * dt * std::pow(fmax_(mid - sY, R(0)), ih);
      if (g > R(0)) hi = mid;
      else lo = mid;
    }
    sNew = R(0.5) * (lo + hi);
  }
  V3<R> bNew = devb * (sNew / sPre) + splat(trb / R(3));
  bNew = vmax(bNew, splat<R>(R(1e-6)));
  R detB = bNew.x * bNew.y * bNew.z;
  bNew = bNew * std::pow(detB, R(-1.0 / 3.0));
  return vsqrt(bNew) * std::pow(J, R(1.0 / 3.0));
}
// NACC, common.js:287-364
template <class R> V3<R> rmNACC(V3<R> sig, const MatR<R>& m, R alphaIn, R& alphaOut) {
  R beta = m.p1, xi = m.p2, Mf = m.p3, mu = m.mu;
  R kappa = R(2.0 / 3.0) * mu + m.lam;
  R alpha = alphaIn;
  V3<R> s3 = safeSig(sig);
  R Jtr = s3.x * s3.y * s3.z;
  V3<R> b2 = s3 * s3;
  R trb = b2.x + b2.y + b2.z;
  V3<R> devb = b2 - splat(trb / R(3));
  V3<R> sHat = mu * std::pow(Jtr, R(-2.0 / 3.0)) * devb;
  R sNorm = length(sHat);
  R q = R(std::sqrt(1.5)) * sNorm;
  R p = R(-0.5) * kappa * (Jtr * Jtr - R(1));
  alpha = clampf(alpha, R(-0.25), R(0.4));
  R p0 = kappa * (R(0.00001) + std::sinh(fmin_(xi * fmax_(-alpha, R(0)), R(4))));
  R b = R(1) + R(2) * beta;
  V3<R> outSig = sig;
  if (p > p0) {
    R Jn = std::sqrt(fmax_(R(-2) * p0 / kappa + R(1), R(1e-6)));
    outSig = splat(std::pow(Jn, R(1.0 / 3.0)));
    alpha = alpha + std::log(Jtr / Jn);
  } else if (p < -beta * p0) {
    R Jn = std::sqrt(fmax_(R(2) * beta * p0 / kappa + R(1), R(1e-6)));
    outSig = splat(std::pow(Jn, R(1.0 / 3.0)));
    alpha = alpha + std::log(Jtr / Jn);
  } else {
    R y = b * q * q + Mf * Mf * (p + beta * p0) * (p - p0);
    if (y > R(1e-4) && sNorm > R(1e-9)) {
      if (p0 > R(1e-4) && p < p0 - R(1e-4) && p > -beta * p0 + R(1e-4)) {
        R pc = (R(1) - beta) * p0 * R(0.5);
        R lenDir = std::sqrt((pc - p) * (pc - p) + (-q) * (-q));
        if (lenDir > R(1e-9)) {
          R Dp = (pc - p) / lenDir;
          R Dq = -q / lenDir;
          R Aq = Mf * Mf * Dp * Dp + b * Dq * Dq;
          R Bq = Mf * Mf * Dp * (R(2) * pc - p0 + beta * p0);
          R Cq = Mf * Mf * (pc + beta * p0) * (pc - p0);
          R disc = Bq * Bq - R(4) * Aq * Cq;
          if (disc > R(0) && std::fabs(Aq) > R(1e-12)) {
            R l1 = (-Bq + std::sqrt(disc)) / (R(2) * Aq);
            R l2 = (-Bq - std::sqrt(disc)) / (R(2) * Aq);
            R px1 = pc + l1 * Dp;
            R px2 = pc + l2 * Dp;
            R px = px1;
            if ((p - pc) * (px2 - pc) > R(0)) px = px2;
            R Jx2 = R(-2) * px / kappa + R(1);
            if (Jx2 > R(1e-8)) {
              R Jx = std::sqrt(Jx2);
              if (Jx > R(1e-4)) alpha = alpha + std::log(Jtr / Jx);
            }
          }
        }
      }
      R qN = Mf * std::sqrt(fmax_(-(p + beta * p0) * (p - p0), R(0)) / b);
      R sNewNorm = qN / R(std::sqrt(1.5));
      V3<R> bNew = (std::pow(Jtr, R(2.0 / 3.0)) / mu) * (sNewNorm / sNorm) * sHat + splat(trb / R(3));
      bNew = vmax(bNew, splat<R>(R(1e-6)));
      outSig = vsqrt(bNew);
    }
  }
  alphaOut = alpha;
  return outSig;
}
// hardenedMat, common.js:366-375
template <class R> MatR<R> hardenedMat(const MatR<R>& m, R state) {
  MatR<R> mm = m;
  if (m.kind == MAT_SNOW) {
    R s = std::exp(fmin_(m.p2 * (R(1) - state), R(5)));
    mm.mu = m.mu * s;
    mm.lam = m.lam * s;
  }
  return mm;
}
// returnMap, common.js:377-396
template <class R> V3<R> returnMap(V3<R> sig, const MatR<R>& m, R state, R dt, R& stateOut) {
  stateOut = state;
  switch (m.kind) {
    case 1u: return rmDruckerPrager(sig, m);
    case 2u: return rmNACC(sig, m, state, stateOut);
    case 3u: return rmVonMises(sig, m);
    case 4u: return rmHerschelBulkley(sig, m, dt);
    case 5u: {
      MatR<R> mm = hardenedMat(m, state);
      V3<R> sNew = vclamp(sig, splat(R(1) - mm.p0), splat(R(1) + mm.p1));
      R jOld = sig.x * sig.y * sig.z;
      R jNew = sNew.x * sNew.y * sNew.z;
      stateOut = clampf(state * jOld / fmax_(jNew, R(1e-6)), R(0.2), R(2));
      return sNew;
    }
    default: return sig;
  }
}

// ------------------------------------------------------- the machine
template <class R> struct V4 { R x, y, z, w; };
template <class R> V3<R> xyz(const V4<R>& a) { return {a.x, a.y, a.z}; }

template <class R> struct Machine {
  Params<R> P;
  uint32_t N;
  V4<R>* pos;
  V4<R>* velA;
  V4<R>* aux;
  M3<R>* F;
  M3<R>* L;
  uint32_t* cellTab;
  uint32_t* sortedIdx;
  std::vector<V4<R>> velB, Sp;  // Sp: 3 vec4 per particle
  V4<R>* velIn;
  V4<R>* velOut;

  uint32_t matOf(uint32_t i) const {
    R w = pos[i].w;
    if (!(w > R(0))) return 0u;
    uint32_t m = (uint32_t)w;
    return m > 7u ? 7u : m;
  }
  bool isSolid(uint32_t mi) const { return P.mats[mi].kind != MAT_WATER; }

  // simkernels.js:62-74
  void rowRange(I3 c, uint32_t& beg, uint32_t& end) const {
    if (c.y < 0 || c.y >= P.dims[1] || c.z < 0 || c.z >= P.dims[2]) { beg = end = 0; return; }
    int x0 = std::max(c.x - 1, 0);
    int x1 = std::min(c.x + 1, P.dims[0] - 1);
    uint32_t c0 = cellIndex(P, I3{x0, c.y, c.z});
    uint32_t c2 = cellIndex(P, I3{x1, c.y, c.z});
    beg = cellTab[c0];
    uint32_t e = P.N;
    if (c2 + 1u < P.numCells) e = cellTab[c2 + 1u];
    end = std::min(e, beg + ROW_CAP);
  }
  template <class Body> void stencil(V3<R> x, Body&& body) const {
    I3 cc = cellCoord(P, x);
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy) {
        uint32_t b0, b1;
        rowRange(I3{cc.x, cc.y + dy, cc.z + dz}, b0, b1);
        for (uint32_t b = b0; b < b1; ++b) body(b);
      }
  }
  R support2() const { return P.support * P.support; }

  // ---- counting sort: simkernels.js:78-147 (serial-atomic semantics)
  void sortAndPredict() {
    std::fill(cellTab, cellTab + P.numCells, 0u);
    std::vector<uint32_t> key(N);
    for (uint32_t i = 0; i < N; ++i) {
      key[i] = cellIndex(P, cellCoord(P, xyz(pos[i])));
      cellTab[key[i]] += 1u;
    }
    uint32_t run = 0;  // scanBlocks + scanApply: inclusive prefix sums
    for (uint32_t c = 0; c < P.numCells; ++c) { run += cellTab[c]; cellTab[c] = run; }
    for (uint32_t i = 0; i < N; ++i) {  // scatter, ascending i
      uint32_t dst = --cellTab[key[i]];
      sortedIdx[dst] = i;
    }
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)N; ++ii) {
      uint32_t i = (uint32_t)ii;
      R Vn = P.V0 * clampf(det(F[i]), R(0.1), R(10));
      aux[i].x = Vn;
      V3<R> g = v3(P.gravity[0], P.gravity[1], P.gravity[2]);
      V3<R> v = xyz(velIn[i]) + g * P.dt;
      velIn[i] = {v.x, v.y, v.z, Vn};
      aux[i].y = R(0);
    }
  }
  // ---- stagePVA/applyPVA/stageF/applyF: simkernels.js:154-186
  void reorder() {
    std::vector<V4<R>> p2(N), v2(N), a2(N);
    std::vector<M3<R>> f2(N);
#pragma omp parallel for schedule(static)
    for (int64_t jj = 0; jj < (int64_t)N; ++jj) {
      uint32_t i = sortedIdx[jj];
      p2[jj] = pos[i]; v2[jj] = velIn[i]; a2[jj] = aux[i]; f2[jj] = F[i];
    }
#pragma omp parallel for schedule(static)
    for (int64_t jj = 0; jj < (int64_t)N; ++jj) {
      pos[jj] = p2[jj]; velIn[jj] = v2[jj]; velOut[jj] = v2[jj]; aux[jj] = a2[jj]; F[jj] = f2[jj];
    }
  }
  // ---- computeL: simkernels.js:189-221
  void computeL() {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t ii = 0; ii < (int64_t)N; ++ii) {
      uint32_t i = (uint32_t)ii;
      V3<R> xi = xyz(pos[i]);
      M3<R> A = mzero<R>();
      stencil(xi, [&](uint32_t b) {
        if (b == i) return;
        V3<R> dxv = xi - xyz(pos[b]);
        if (dot(dxv, dxv) < support2()) {
          V3<R> g = kernelGradW(P, dxv);
          V3<R> r = xyz(pos[b]) - xi;
          M3<R> o = {{g * r.x, g * r.y, g * r.z}};
          A = madd(A, mscale(o, velIn[b].w));
        }
      });
      SVD<R> s = svd3(A);
      const R tol = R(0.2);
      V3<R> inv = splat<R>(0);
      if (std::fabs(s.sig.x) > tol) inv.x = R(1) / s.sig.x;
      if (std::fabs(s.sig.y) > tol) inv.y = R(1) / s.sig.y;
      if (std::fabs(s.sig.z) > tol) inv.z = R(1) / s.sig.z;
      L[i] = diagMul(s.V, inv, s.U);
    }
  }
  // ---- velocityGradient: simkernels.js:224-245
  M3<R> velocityGradient(uint32_t i, V3<R> xi) const {
    M3<R> G = mzero<R>();
    const M3<R>& Li = L[i];
    V3<R> vi = xyz(velIn[i]);
    stencil(xi, [&](uint32_t b) {
      if (b == i || !isSolid(matOf(b))) return;
      V3<R> dxv = xi - xyz(pos[b]);
      if (dot(dxv, dxv) < support2()) {
        V3<R> gt = mul(Li, kernelGradW(P, dxv));
        V4<R> vb = velIn[b];
        V3<R> dv = (xyz(vb) - vi) * vb.w;
        G = madd(G, M3<R>{{dv * gt.x, dv * gt.y, dv * gt.z}});
      }
    });
    return G;
  }
  void storeSp(uint32_t i, const M3<R>& m, V3<R> s) {
    Sp[3 * i] = {m.c[0].x, m.c[0].y, m.c[0].z, s.x};
    Sp[3 * i + 1] = {m.c[1].x, m.c[1].y, m.c[1].z, s.y};
    Sp[3 * i + 2] = {m.c[2].x, m.c[2].y, m.c[2].z, s.z};
  }
  // ---- solveA: simkernels.js:248-309
  void solveA() {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t ii = 0; ii < (int64_t)N; ++ii) {
      uint32_t i = (uint32_t)ii;
      uint32_t mi = matOf(i);
      if (!isSolid(mi)) { storeSp(i, mzero<R>(), splat<R>(0)); continue; }
      MatR<R> m = hardenedMat(P.mats[mi], aux[i].z);
      V3<R> xi = xyz(pos[i]);
      M3<R> Fn = F[i];
      M3<R> gradV = velocityGradient(i, xi);
      M3<R> Ftr = mul(madd(mident<R>(), mscale(gradV, P.dt)), Fn);
      SVD<R> sv = svd3(Ftr);
      R st;
      V3<R> sig = returnMap(sv.sig, m, aux[i].z, P.dt, st);
      R psi = stvkPsi(sig, m.mu, m.lam);
      R C = std::sqrt(fmax_(R(2) * psi, R(0)));
      if (C < R(1e-7)) { storeSp(i, mzero<R>(), splat<R>(0)); continue; }
      V3<R> dpsi = stvkDPsi(sig, m.mu, m.lam);
      M3<R> Pk = diagMul(sv.U, dpsi / C, sv.V);
      M3<R> GL = mul(mul(Pk, transpose(Fn)), L[i]);
      R denom = R(0), cdot = R(0);
      V3<R> sgrad = splat<R>(0);
      stencil(xi, [&](uint32_t b) {
        if (b == i || !isSolid(matOf(b))) return;
        V3<R> dxv = xi - xyz(pos[b]);
        if (dot(dxv, dxv) < support2()) {
          V4<R> vb = velIn[b];
          V3<R> gb = vb.w * mul(GL, kernelGradW(P, dxv));
          denom = denom + dot(gb, gb) / P.mats[matOf(b)].mass;
          sgrad = sgrad - gb;
          cdot = cdot + dot(gb, xyz(vb));
        }
      });
      denom = denom + dot(sgrad, sgrad) / m.mass;
      cdot = cdot + dot(sgrad, xyz(velIn[i]));
      R alphaT = (R(1) / P.V0) / (P.dt * P.dt);
      R g = P.kDamp;
      R dlam = P.omega * (-C - alphaT * aux[i].y - g * P.dt * cdot) / ((R(1) + g) * denom + alphaT);
      aux[i].y = aux[i].y + dlam;
      storeSp(i, mscale(GL, dlam), sgrad * dlam);
    }
  }
  // ---- applyBoundary: simkernels.js:369-404
  V3<R> applyBoundary(V3<R> xcIn, V3<R> vIn, V3<R> xn, R fric) const {
    V3<R> vv = vIn, xq = xcIn;
    for (int k = 0; k < 3; ++k) {
      R lo = P.domainMin[k], hi = P.domainMax[k];
      if (xq[k] < lo || xq[k] > hi) {
        R bound = xq[k] < lo ? lo : hi;
        R vnNew = (bound - xn[k]) / P.dt;
        R dvn = std::fabs(vnNew - vv[k]);
        V3<R> vt = vv;
        vt[k] = R(0);
        R vtl = length(vt);
        if (vtl > R(1e-9)) {
          R drop = fmin_(fric * dvn, vtl);
          vv = vv - vt / vtl * drop;
        }
        vv[k] = vnNew;
        xq = xn + P.dt * vv;
      }
    }
    if (P.colliderActive > R(0.5)) {
      V3<R> cp = v3(P.colliderPos[0], P.colliderPos[1], P.colliderPos[2]);
      V3<R> cv = v3(P.colliderVel[0], P.colliderVel[1], P.colliderVel[2]);
      V3<R> d = xq - cp;
      R dist = length(d);
      if (dist < P.colliderR && dist > R(1e-9)) {
        V3<R> n = d / dist;
        R vOut = dot(vv - cv, n);
        R vGoal = fmin_((P.colliderR - dist) / P.dt, R(0.6));
        if (vOut < vGoal) vv = vv + n * (vGoal - vOut);
      }
    }
    return vv;
  }
  // ---- solveB: simkernels.js:315-366
  void solveB() {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t ii = 0; ii < (int64_t)N; ++ii) {
      uint32_t i = (uint32_t)ii;
      uint32_t mi = matOf(i);
      V3<R> dv = splat<R>(0), corr = splat<R>(0);
      V3<R> xi = xyz(pos[i]);
      const MatR<R>& m = P.mats[mi];
      if (isSolid(mi)) {
        dv = v3(Sp[3 * i].w, Sp[3 * i + 1].w, Sp[3 * i + 2].w);
        R Vi = velIn[i].w;
        V3<R> xci = xi + P.dt * xyz(velIn[i]);
        R minD = R(0.75) * P.h;
        stencil(xi, [&](uint32_t b) {
          if (b == i || !isSolid(matOf(b))) return;
          V3<R> pb = xyz(pos[b]);
          V3<R> dxp = pb - xi;
          if (dot(dxp, dxp) < support2()) {
            M3<R> Sb = {{xyz(Sp[3 * b]), xyz(Sp[3 * b + 1]), xyz(Sp[3 * b + 2])}};
            dv = dv + Vi * mul(Sb, kernelGradW(P, dxp));
            V3<R> xcb = pb + P.dt * xyz(velIn[b]);
            V3<R> dxc = xci - xcb;
            R dist = length(dxc);
            if (dist < minD && dist > R(1e-9)) {
              R mb = P.mats[matOf(b)].mass;
              R w = mb / (m.mass + mb);
              corr = corr + dxc / dist * ((minD - dist) * w);
            }
          }
        });
      }
      V3<R> dvv = dv / (m.mass * P.dt);
      R dvl = length(dvv);
      R dvCap = R(0.2) * P.support / P.dt;
      if (dvl > dvCap) dvv = dvv * (dvCap / dvl);
      V3<R> v = xyz(velIn[i]) + dvv + corr * (P.contactOmega / P.dt);
      v = applyBoundary(xi + P.dt * v, v, xi, m.boundFriction);
      velOut[i] = {v.x, v.y, v.z, velIn[i].w};
    }
  }
  // ---- pbfA: simkernels.js:407-439
  void pbfA() {
    const R w00 = kernelPoly6(P, R(0));
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t ii = 0; ii < (int64_t)N; ++ii) {
      uint32_t i = (uint32_t)ii;
      if (isSolid(matOf(i))) { aux[i].w = R(0); continue; }
      const MatR<R>& m = P.mats[matOf(i)];
      R rho0 = m.density;
      V3<R> xn = xyz(pos[i]);
      V3<R> xci = xn + P.dt * xyz(velIn[i]);
      R rho = m.mass * w00;
      V3<R> gradSum = splat<R>(0);
      R grad2 = R(0);
      stencil(xn, [&](uint32_t b) {
        if (b == i) return;
        V3<R> xcb = xyz(pos[b]) + P.dt * xyz(velIn[b]);
        V3<R> dxv = xci - xcb;
        if (dot(dxv, dxv) < support2()) {
          R mb = P.mats[matOf(b)].mass;
          rho = rho + mb * kernelPoly6(P, length(dxv));
          V3<R> g = kernelSpikyGrad(P, dxv) * (mb / rho0);
          gradSum = gradSum + g;
          grad2 = grad2 + dot(g, g);
        }
      });
      R C = fmax_(rho / rho0 - R(1), R(0));
      aux[i].w = -C / (grad2 + dot(gradSum, gradSum) + P.pbfEps);
    }
  }
  // ---- pbfB: simkernels.js:441-477
  void pbfB() {
    const R w0 = kernelPoly6(P, R(0.2) * P.support);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t ii = 0; ii < (int64_t)N; ++ii) {
      uint32_t i = (uint32_t)ii;
      uint32_t mi = matOf(i);
      V3<R> xn = xyz(pos[i]);
      V3<R> xci = xn + P.dt * xyz(velIn[i]);
      V3<R> dp = splat<R>(0);
      R li = aux[i].w;
      bool iAmWater = !isSolid(mi);
      stencil(xn, [&](uint32_t b) {
        if (b == i) return;
        bool bWater = !isSolid(matOf(b));
        if (!(iAmWater || bWater)) return;
        V3<R> xcb = xyz(pos[b]) + P.dt * xyz(velIn[b]);
        V3<R> dxv = xci - xcb;
        if (dot(dxv, dxv) < support2()) {
          const MatR<R>& mw = P.mats[bWater ? matOf(b) : mi];
          R lb = aux[b].w;
          R w = kernelPoly6(P, length(dxv));
          R sCorr = -P.sCorrK * std::pow(w / fmax_(w0, R(1e-12)), R(4));
          dp = dp + (li + lb + sCorr) * kernelSpikyGrad(P, dxv) * (mw.mass / mw.density);
        }
      });
      R scale = iAmWater ? R(1) : R(0.5);
      V3<R> v = xyz(velIn[i]) + dp * (scale / P.dt);
      velOut[i] = {v.x, v.y, v.z, velIn[i].w};
    }
  }
  // ---- xsph: simkernels.js:480-507
  void xsph() {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t ii = 0; ii < (int64_t)N; ++ii) {
      uint32_t i = (uint32_t)ii;
      V3<R> xi = xyz(pos[i]);
      V3<R> vi = xyz(velIn[i]);
      bool iSolid = isSolid(matOf(i));
      V3<R> acc = splat<R>(0);
      stencil(xi, [&](uint32_t b) {
        if (b == i || isSolid(matOf(b)) != iSolid) return;
        V3<R> dxv = xi - xyz(pos[b]);
        if (dot(dxv, dxv) < support2()) {
          V4<R> vb = velIn[b];
          acc = acc + vb.w * (xyz(vb) - vi) * kernelW(P, length(dxv));
        }
      });
      R c = P.xsphC;
      if (!iSolid) c = P.xsphC * R(10);
      V3<R> v = vi + c * acc;
      velOut[i] = {v.x, v.y, v.z, velIn[i].w};
    }
  }
  // ---- updateF: simkernels.js:510-525
  void updateF() {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t ii = 0; ii < (int64_t)N; ++ii) {
      uint32_t i = (uint32_t)ii;
      uint32_t mi = matOf(i);
      if (!isSolid(mi)) continue;
      MatR<R> m = hardenedMat(P.mats[mi], aux[i].z);
      M3<R> gradV = velocityGradient(i, xyz(pos[i]));
      M3<R> Ftr = mul(madd(mident<R>(), mscale(gradV, P.dt)), F[i]);
      SVD<R> sv = svd3(Ftr);
      R st;
      V3<R> sig = returnMap(sv.sig, m, aux[i].z, P.dt, st);
      F[i] = diagMul(sv.U, safeSig(sig), sv.V);
      aux[i].z = st;
    }
  }
  // ---- integrate: simkernels.js:528-542
  void integrate() {
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)N; ++ii) {
      uint32_t i = (uint32_t)ii;
      V3<R> v = xyz(velIn[i]);
      R vmax = R(0.45) * P.support / P.dt;
      R vl = length(v);
      if (vl > vmax) v = v * (vmax / vl);
      velIn[i] = {v.x, v.y, v.z, velIn[i].w};
      V3<R> x = xyz(pos[i]) + P.dt * v;
      x = vclamp(x, v3(P.domainMin[0], P.domainMin[1], P.domainMin[2]),
                 v3(P.domainMax[0], P.domainMax[1], P.domainMax[2]));
      pos[i] = {x.x, x.y, x.z, pos[i].w};
    }
  }
  // ---- encodeSubstep: sim.js:220-272. pbfIterations < 0 means "every
  // iteration" (the reference's interleave); otherwise PBF runs on the first
  // pbfIterations XPBI iterations.
  void substep(int iterations, bool hasWater, int pbfIterations) {
    velIn = velA;
    velOut = velB.data();
    bool flip = false;
    auto swap = [&]() { std::swap(velIn, velOut); flip = !flip; };
    sortAndPredict();
    reorder();
    computeL();
    for (int k = 0; k < iterations; ++k) {
      solveA();
      solveB();
      swap();
      if (hasWater && (pbfIterations < 0 || k < pbfIterations)) {
        pbfA();
        pbfB();
        swap();
      }
    }
    xsph();
    swap();
    updateF();
    integrate();
    if (flip) std::copy(velB.begin(), velB.end(), velA);
  }
};

template <class R>
int run_substeps(const uint32_t* params, const uint32_t* mats, uint32_t n, R* pos, R* vel, R* F12, R* L12,
                 R* aux, uint32_t* sortedIdx, uint32_t* cellTab, int iterations, int hasWater,
                 int pbfIterations, int substeps, int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  Machine<R> M;
  M.P = decode<R>(params, mats);
  if (M.P.N != n) return -1;
  M.N = n;
  M.pos = reinterpret_cast<V4<R>*>(pos);
  M.velA = reinterpret_cast<V4<R>*>(vel);
  M.aux = reinterpret_cast<V4<R>*>(aux);
  M.cellTab = cellTab;
  M.sortedIdx = sortedIdx;
  std::vector<M3<R>> F(n), L(n);
  for (uint32_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      F[i].c[c] = v3(F12[12 * i + 4 * c], F12[12 * i + 4 * c + 1], F12[12 * i + 4 * c + 2]);
      L[i].c[c] = v3(L12[12 * i + 4 * c], L12[12 * i + 4 * c + 1], L12[12 * i + 4 * c + 2]);
    }
  M.F = F.data();
  M.L = L.data();
  M.velB.assign(n, V4<R>{0, 0, 0, 0});
  M.Sp.assign(3 * (size_t)n, V4<R>{0, 0, 0, 0});
  for (int s = 0; s < substeps; ++s) M.substep(iterations, hasWater != 0, pbfIterations);
  for (uint32_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      F12[12 * i + 4 * c] = F[i].c[c].x; F12[12 * i + 4 * c + 1] = F[i].c[c].y;
      F12[12 * i + 4 * c + 2] = F[i].c[c].z; F12[12 * i + 4 * c + 3] = R(0);
      L12[12 * i + 4 * c] = L[i].c[c].x; L12[12 * i + 4 * c + 1] = L[i].c[c].y;
      L12[12 * i + 4 * c + 2] = L[i].c[c].z; L12[12 * i + 4 * c + 3] = R(0);
    }
  return 0;
}

}  // namespace

extern "C" {

// One or more substeps in f32 on the reference layouts (sim.js:32-82): pos and
// vel are vec4 x N, F and L are mat3x3f x N (3 columns padded to vec4, 12
// floats), aux is vec4 x N (Vn, lambda, state, pbf lambda). sortedIdx (N) and
// cellTab (numCells) receive the last substep's permutation and cell starts.
int xo_substep_f32(const uint32_t* params, const uint32_t* mats, uint32_t n, float* pos, float* vel, float* F12,
                   float* L12, float* aux, uint32_t* sortedIdx, uint32_t* cellTab, int iterations, int hasWater,
                   int pbfIterations, int substeps, int threads) {
  return run_substeps<float>(params, mats, n, pos, vel, F12, L12, aux, sortedIdx, cellTab, iterations, hasWater,
                             pbfIterations, substeps, threads);
}

// Same substep in f64 arithmetic on f64 state arrays (callers widen the f32
// state they want to compare against).
int xo_substep_f64(const uint32_t* params, const uint32_t* mats, uint32_t n, double* pos, double* vel,
                   double* F12, double* L12, double* aux, uint32_t* sortedIdx, uint32_t* cellTab, int iterations,
                   int hasWater, int pbfIterations, int substeps, int threads) {
  return run_substeps<double>(params, mats, n, pos, vel, F12, L12, aux, sortedIdx, cellTab, iterations, hasWater,
                              pbfIterations, substeps, threads);
}

// ---- pieces of common.js exposed for known-answer tests (f32 and f64)
int xo_svd3_f32(const float* F9, float* U9, float* sig3, float* V9) {
  M3<float> F;
  for (int c = 0; c < 3; ++c) F.c[c] = v3(F9[3 * c], F9[3 * c + 1], F9[3 * c + 2]);
  SVD<float> s = svd3(F);
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) { U9[3 * c + r] = s.U.c[c][r]; V9[3 * c + r] = s.V.c[c][r]; }
  sig3[0] = s.sig.x; sig3[1] = s.sig.y; sig3[2] = s.sig.z;
  return 0;
}

// Return map on n singular-value triples with material words mat16 (one
// Material as packed by sim.js:84-99); state in/out per triple.
int xo_return_map_f64(const uint32_t* mat16, double dt, uint32_t n, const double* sig, double* out,
                      double* state) {
  uint32_t mats[128] = {0};
  std::memcpy(mats, mat16, 64);
  uint32_t params[64] = {0};
  Params<double> P = decode<double>(params, mats);
  for (uint32_t i = 0; i < n; ++i) {
    double st;
    V3<double> r = returnMap(v3(sig[3 * i], sig[3 * i + 1], sig[3 * i + 2]), P.mats[0], state[i], dt, st);
    out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
    state[i] = st;
  }
  return 0;
}
int xo_return_map_f32(const uint32_t* mat16, float dt, uint32_t n, const float* sig, float* out, float* state) {
  uint32_t mats[128] = {0};
  std::memcpy(mats, mat16, 64);
  uint32_t params[64] = {0};
  Params<float> P = decode<float>(params, mats);
  for (uint32_t i = 0; i < n; ++i) {
    float st;
    V3<float> r = returnMap(v3(sig[3 * i], sig[3 * i + 1], sig[3 * i + 2]), P.mats[0], state[i], dt, st);
    out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
    state[i] = st;
  }
  return 0;
}
// StVK-Hencky energy and its sigma-gradient (common.js:190-201), f64.
int xo_stvk_f64(double mu, double lam, uint32_t n, const double* sig, double* psi, double* dpsi) {
  for (uint32_t i = 0; i < n; ++i) {
    V3<double> s = v3(sig[3 * i], sig[3 * i + 1], sig[3 * i + 2]);
    psi[i] = stvkPsi(s, mu, lam);
    V3<double> d = stvkDPsi(s, mu, lam);
    dpsi[3 * i] = d.x; dpsi[3 * i + 1] = d.y; dpsi[3 * i + 2] = d.z;
  }
  return 0;
}
// Wendland C2 value and gradient for a given h (common.js:63-79), f64.
int xo_kernel_f64(double h, uint32_t n, const double* dx3, double* w, double* gw3) {
  uint32_t params[64] = {0};
  uint32_t mats[128] = {0};
  Params<double> P = decode<double>(params, mats);
  P.h = h;
  P.support = 2 * h;
  for (uint32_t i = 0; i < n; ++i) {
    V3<double> d = v3(dx3[3 * i], dx3[3 * i + 1], dx3[3 * i + 2]);
    w[i] = kernelW(P, length(d));
    V3<double> g = kernelGradW(P, d);
    gw3[3 * i] = g.x; gw3[3 * i + 1] = g.y; gw3[3 * i + 2] = g.z;
  }
  return 0;
}
// Poly6 value and spiky gradient with H = 2h (common.js:81-94), f64.
int xo_pbf_kernels_f64(double h, uint32_t n, const double* dx3, double* w, double* gw3) {
  uint32_t params[64] = {0};
  uint32_t mats[128] = {0};
  Params<double> P = decode<double>(params, mats);
  P.h = h;
  P.support = 2 * h;
  for (uint32_t i = 0; i < n; ++i) {
    V3<double> d = v3(dx3[3 * i], dx3[3 * i + 1], dx3[3 * i + 2]);
    w[i] = kernelPoly6(P, length(d));
    V3<double> g = kernelSpikyGrad(P, d);
    gw3[3 * i] = g.x; gw3[3 * i + 1] = g.y; gw3[3 * i + 2] = g.z;
  }
  return 0;
}

}  // extern "C"
