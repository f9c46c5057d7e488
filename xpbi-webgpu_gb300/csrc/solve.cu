// Neighbour-gather kernels of the XPBI substep, one thread per particle slot
// in cell order. Each restates one compute entry point of
// web/js/shaders/simkernels.js (cited per kernel).
//
// Neighbour lists. Positions do not move between the reorder and the final
// update, so the set of in-support neighbours (b != i, |x_i - x_b|^2 <
// support^2) is the same for computeL, every solveA / solveB iteration, xsph
// and updateF. computeL walks the reference stencil once (dz outer, dy inner,
// candidates ascending over the row-merged range of three x-adjacent cells,
// capped at 384, simkernels.js:62-74) and records the in-support neighbours in
// that order, so every later pass sums over exactly the reference's terms in
// the reference's order without rescanning ~216 candidates per particle.
// Lists that do not fit kNbrCap fall back to the stencil walk.
//
// PBF passes test predicted positions x + dt v, which change every
// iteration: pbfA walks the stencil once per pass, records the predicted
// neighbours, and both PBF kernels then iterate that record.
//
// Scans are two-phase: a branch-light candidate test that only records
// indices, then a uniform pass over the record; list loops issue the gathers
// of entry k+1 before the arithmetic of entry k. (The candidate-scan
// versions ran with ~14 of 32 lanes active and stalled on gathers.)
//
// Sorted records carry the water flag in the sign bit of pos.w (pos.w is
// material index + colour seed >= 0, so fabsf restores it exactly).
//
// Batched handles: every slot belongs to one scene (sceneOf); its grid, cell
// table range, uniforms and material table come from that scene, and a
// neighbour stencil never leaves the scene's own cells. Passes beyond a
// scene's iteration budget copy velIn to velOut so the shared ping-pong
// parity stays consistent for every scene.
#include <algorithm>

#include "xpbi_math.cuh"

namespace xpbi {

namespace {

constexpr int kThreads = 128;

// Launch bounds of the stencil kernels: defining XPBI_MINB_<KERNEL> at build
// time asks the register allocator for that many resident CTAs per SM
// (trading registers for occupancy); otherwise only the block size is fixed.
#define XPBI_LB_DEFAULT __launch_bounds__(kThreads)
#ifdef XPBI_MINB_COMPUTEL
#define XPBI_LB_COMPUTEL __launch_bounds__(kThreads, XPBI_MINB_COMPUTEL)
#else
#define XPBI_LB_COMPUTEL XPBI_LB_DEFAULT
#endif
// computeL with the stored constraint and features (the learned solve) at
// 7 CTAs per SM (72 registers): 1.36 ms per 4M-particle substep against
// 1.56 ms with the allocator's choice (5 CTAs).
#ifndef XPBI_MINB_COMPUTEL_FEATURES
#define XPBI_MINB_COMPUTEL_FEATURES 7
#endif
#define XPBI_LB_COMPUTEL_FEATURES __launch_bounds__(kThreads, XPBI_MINB_COMPUTEL_FEATURES)
// solveA and solveB are compiled in several launch shapes — the block size
// and the minimum resident CTAs per SM asked of the register allocator (0 =
// its own choice) — and xpbi_autotune picks one per handle by timing them on
// its data. Entry 0 is the default: for solveA 8 CTAs of 128 per SM (64
// registers; the constraint's per-particle tail is a separately compiled
// function) — 0.396 ms per launch on the 4M-particle dam-breach mix against
// 0.417 at 7 CTAs, 0.421 at 9, 0.438 at 10 and 0.58 at 5, and the best or
// within 1% on the 256-scene batch, the snowball and the sand column; for
// solveB the allocator's choice (80 registers) beat every cap. The 64- and
// 256-thread shapes keep an entry's occupancy with other block sizes.
constexpr int kSolveAMinB[kSolveAVariants] = {8, 6, 5, 7, 14, 4};
constexpr int kSolveABlock[kSolveAVariants] = {128, 128, 128, 128, 64, 256};
constexpr int kSolveBMinB[kSolveBVariants] = {0, 7, 5, 0, 0};
constexpr int kSolveBBlock[kSolveBVariants] = {128, 128, 128, 64, 256};
#ifdef XPBI_MINB_PBF
#define XPBI_LB_PBF __launch_bounds__(kThreads, XPBI_MINB_PBF)
#else
#define XPBI_LB_PBF XPBI_LB_DEFAULT
#endif
#ifdef XPBI_MINB_UPDATE
#define XPBI_LB_UPDATE __launch_bounds__(kThreads, XPBI_MINB_UPDATE)
#else
#define XPBI_LB_UPDATE XPBI_LB_DEFAULT
#endif

struct Ctx {
  const SceneDev* __restrict__ scene;
  const MatDev* __restrict__ mats;  // this scene's 8 materials
};

__device__ __forceinline__ Ctx ctxOf(const Bufs& b, uint32_t i) {
  const uint32_t s = b.S > 1 ? (uint32_t)b.sceneOf[i] : 0u;
  const SceneDev* S = b.scenes + s;
  return Ctx{S, b.mats + S->matBase};
}

// material index stored as a float value in pos.w (simkernels.js:41-44)
__device__ __forceinline__ uint32_t matOfW(float w) {
  w = fabsf(w);
  if (!(w > 0.f)) return 0u;
  const uint32_t m = (uint32_t)w;
  return m > 7u ? 7u : m;
}
__device__ __forceinline__ bool waterW(float w) { return signbit(w); }

struct PV {
  float4 p, v;
};

template <class T>
__device__ __forceinline__ T ldg(const T* p) {
  return __ldg(p);
}

// Stencil walk over the 9 row-merged ranges (simkernels.js:62-74):
// row(beg, end) is called per in-range row.
template <class Row>
__device__ __forceinline__ void forRows(const SceneDev& S, const uint32_t* __restrict__ cellStart, V3 x, Row&& row) {
  const I3 cc = cellCoord(S, x);
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
      const uint32_t beg = __ldg(cellStart + c0);
      const uint32_t end = min(__ldg(cellStart + c2 + 1), beg + kRowCap);
      row(beg, end);
    }
  }
}

// A particle's list occupies kNbrCap consecutive words (16-byte aligned) and
// is read four entries per load, one load ahead; the gather of entry k+1 is
// issued before the body of entry k runs.
__device__ __forceinline__ uint32_t lane4(const uint4& q, uint32_t s) {
  return s == 0u ? q.x : (s == 1u ? q.y : (s == 2u ? q.z : q.w));
}

// kRaw: gather() receives the raw entry (index | water bit), e.g. to skip
// the loads of entries the body ignores.
template <bool kRaw = false, class Gather, class Body>
__device__ __forceinline__ void forList(const uint32_t* __restrict__ list, uint32_t cnt, Gather&& gather,
                                        Body&& body) {
  if (cnt == 0) return;
  const uint4* __restrict__ L = reinterpret_cast<const uint4*>(list);
  uint4 cur = __ldg(L);
  uint4 nxt = cnt > 4u ? __ldg(L + 1) : cur;
  uint32_t e = cur.x;
  auto d = gather(kRaw ? e : e & ~kWaterBit);
#pragma unroll 1
  for (uint32_t k = 1; k < cnt; ++k) {
    const uint32_t sl = k & 3u;
    if (sl == 0u) {
      cur = nxt;
      if (k + 4u < cnt) nxt = __ldg(L + (k >> 2) + 1);
    }
    const uint32_t en = lane4(cur, sl);
    auto dn = gather(kRaw ? en : en & ~kWaterBit);
    body(e & ~kWaterBit, (e & kWaterBit) != 0u, d);
    e = en;
    d = dn;
  }
  body(e & ~kWaterBit, (e & kWaterBit) != 0u, d);
}

__device__ __forceinline__ uint32_t* listOf(uint32_t* base, uint32_t i) { return base + (size_t)i * kNbrCap; }

// Keeps every recorded neighbour.
struct KeepAll {
  __device__ __forceinline__ bool operator()(uint32_t) const { return true; }
};

// In-support neighbours of slot i in stencil order: body(j, jIsWater, data).
// keep(entry) (index | water bit) false: the body will ignore that neighbour,
// so its data is not loaded (the body receives a zero-initialised value).
template <class Gather, class Body, class Keep = KeepAll>
__device__ __forceinline__ void forNbrs(const Bufs& b, const Ctx& cx, uint32_t i, V3 xi, Gather&& gather,
                                        Body&& body, Keep keep = Keep{}) {
  const uint32_t cnt = b.nbrCount[i];
  if (cnt != kNbrOverflow) {
    forList<true>(listOf(b.nbr, i), cnt,
                  [&](uint32_t e) {
                    using T = decltype(gather(0u));
                    return keep(e) ? gather(e & ~kWaterBit) : T{};
                  },
                  body);
  } else {
    const SceneDev& S = *cx.scene;
    forRows(S, b.cellStart, xi, [&](uint32_t beg, uint32_t end) {
#pragma unroll 1
      for (uint32_t j = beg; j < end; ++j) {
        if (j == i) continue;
        const float4 pj = ldg(b.posS + j);
        const V3 d = xi - xyz(pj);
        if (dot(d, d) < S.support2) body(j, waterW(pj.w), gather(j));
      }
    });
  }
}

// Several lanes per slot (small scenes): the G lanes of slot i are
// consecutive in the warp; lane `lane` visits the list entries k with
// k % G == lane (each group of four entries is one load, shared by the
// lanes), or on the overflow walk every G-th candidate of each row. Each
// lane accumulates a partial sum; laneSum adds them over the group.
template <int G, class Gather, class Body, class Keep = KeepAll>
__device__ __forceinline__ void forNbrsLanes(const Bufs& b, const Ctx& cx, uint32_t i, V3 xi, uint32_t lane,
                                             Gather&& gather, Body&& body, Keep keep = Keep{}) {
  static_assert(G == 1 || G == 2 || G == 4, "one, two or four lanes per slot");
  if constexpr (G == 1) {
    (void)lane;
    forNbrs(b, cx, i, xi, gather, body, keep);
  } else {
    const uint32_t cnt = b.nbrCount[i];
    if (cnt != kNbrOverflow) {
      const uint4* __restrict__ L = reinterpret_cast<const uint4*>(listOf(b.nbr, i));
      const uint32_t groups = (cnt + 3u) >> 2;
#pragma unroll 1
      for (uint32_t q = 0; q < groups; ++q) {
        const uint4 grp = __ldg(L + q);
#pragma unroll
        for (uint32_t s = lane; s < 4u; s += G) {
          const uint32_t e = lane4(grp, s);
          if (4u * q + s < cnt && keep(e)) body(e & ~kWaterBit, (e & kWaterBit) != 0u, gather(e & ~kWaterBit));
        }
      }
    } else {
      const SceneDev& S = *cx.scene;
      forRows(S, b.cellStart, xi, [&](uint32_t beg, uint32_t end) {
#pragma unroll 1
        for (uint32_t j = beg + lane; j < end; j += G) {
          if (j == i) continue;
          const float4 pj = ldg(b.posS + j);
          const V3 d = xi - xyz(pj);
          if (dot(d, d) < S.support2) body(j, waterW(pj.w), gather(j));
        }
      });
    }
  }
}

template <int G>
__device__ __forceinline__ float laneSum(float v) {
  if constexpr (G == 2) {
    const unsigned group = 0x3u << (threadIdx.x & 30u);  // warp lanes 2p, 2p+1
    v += __shfl_xor_sync(group, v, 1);
  } else if constexpr (G == 4) {
    const unsigned group = 0xFu << (threadIdx.x & 28u);  // warp lanes 4p .. 4p+3
    v += __shfl_xor_sync(group, v, 1);
    v += __shfl_xor_sync(group, v, 2);
  }
  return v;
}
template <int G>
__device__ __forceinline__ V3 laneSum(V3 v) {
  return v3(laneSum<G>(v.x), laneSum<G>(v.y), laneSum<G>(v.z));
}

// Records, in stencil order, the candidates j != i of the rows around `x`
// whose test(j) holds: list entry j | water bit from flag(j).
template <class Test>
__device__ __forceinline__ uint32_t recordCandidates(const SceneDev& S, const uint32_t* __restrict__ cellStart, V3 x,
                                                     uint32_t i, uint32_t* __restrict__ out, Test&& test) {
  uint32_t cnt = 0;
  forRows(S, cellStart, x, [&](uint32_t beg, uint32_t end) {
#pragma unroll 4
    for (uint32_t j = beg; j < end; ++j) {
      uint32_t e;
      const bool ok = test(j, e) && j != i;
      // past the capacity the last slot is overwritten: such a list is
      // marked as overflowed and never read
      if (ok) out[min(cnt, kNbrCap - 1u)] = e;
      cnt += ok ? 1u : 0u;
    }
  });
  return cnt;
}

// A += V_b (v_b - v_i) g_b^T, the constraint sweep's velocity sum, with every
// rounding explicit: solveA's sweep and computeL's (which stores iteration
// 0's constraint for it) form the same bits whatever the compiler would
// fuse around them.
__device__ __forceinline__ void addVelSum(M3& A, const float4& vb, V3 vi, V3 g) {
  const float dx = __fmul_rn(__fsub_rn(vb.x, vi.x), vb.w);
  const float dy = __fmul_rn(__fsub_rn(vb.y, vi.y), vb.w);
  const float dz = __fmul_rn(__fsub_rn(vb.z, vi.z), vb.w);
  const float gc[3] = {g.x, g.y, g.z};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    A.c[c].x = __fmaf_rn(dx, gc[c], A.c[c].x);
    A.c[c].y = __fmaf_rn(dy, gc[c], A.c[c].y);
    A.c[c].z = __fmaf_rn(dz, gc[c], A.c[c].z);
  }
}

// ---------------------------------------------------------------- computeL
// L of slot i (simkernels.js:198-220) over its recorded neighbours: the
// SVD pseudo-inverse of sum V_b (grad W_b) (x_b - x_i)^T. For a solid
// (kSolid) the same sweep also forms the sums of the constraint passes that
// no velocity enters — s = sum V_b g_b, P = sum (V_b^2 / m_b) g_b g_b^T and
// the solid neighbour count, over the solid neighbours in list order — and
// stores them in sgP for every iteration of the substep. With kVel (a solid,
// at the velocities iteration 0 starts from) the sweep also forms that
// iteration's velocity sum Av = sum V_b (v_b - v_i) g_b^T over the solid
// neighbours in list order — the constraint sweep's own expression — and
// hands the sums and L to the caller.
struct SweepSums {
  M3 Av, L;
  V3 sg;
  float p00, p11, p22, p01, p02, p12, cnt;
};
template <bool kSolid, bool kVel = false>
__device__ __forceinline__ void bonetLok(const Bufs& b, const Ctx& cx, uint32_t i, V3 xi, SweepSums* out = nullptr) {
  static_assert(kSolid || !kVel, "the velocity sum is a solid's");
  const SceneDev& S = *cx.scene;
  const float4* __restrict__ posS = b.posS;
  const float4* __restrict__ velIn = b.velS[0];  // V^n (.w), which no pass changes; with kVel also v
  M3 A = mzero(), Av = mzero();
  V3 sg = splat(0.f);
  V3 vi = splat(0.f);
  if constexpr (kVel) vi = xyz(velIn[i]);
  float p00 = 0.f, p11 = 0.f, p22 = 0.f, p01 = 0.f, p02 = 0.f, p12 = 0.f, cnt = 0.f;
  forNbrs(b, cx, i, xi, [&](uint32_t j) { return PV{ldg(posS + j), ldg(velIn + j)}; },
          [&](uint32_t, bool water, const PV& d) {
            const V3 pb = xyz(d.p);
            const V3 g = gradWFast(S, xi - pb);
            const V3 r = pb - xi;
            // A += V_b g r^T with every rounding explicit, so the two
            // instances (with and without the sums below) form the same L
            const float Vb0 = d.v.w;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              A.c[c].x = __fmaf_rn(__fmul_rn(g.x, r[c]), Vb0, A.c[c].x);
              A.c[c].y = __fmaf_rn(__fmul_rn(g.y, r[c]), Vb0, A.c[c].y);
              A.c[c].z = __fmaf_rn(__fmul_rn(g.z, r[c]), Vb0, A.c[c].z);
            }
            if (kSolid && !water) {
              if constexpr (kVel) addVelSum(Av, d.v, vi, g);
              const float Vb = d.v.w;
              sg = sg + g * Vb;
              const float c = Vb * Vb / cx.mats[matOfW(d.p.w)].mass;
              const V3 cg = g * c;
              p00 += cg.x * g.x;
              p11 += cg.y * g.y;
              p22 += cg.z * g.z;
              p01 += cg.x * g.y;
              p02 += cg.x * g.z;
              p12 += cg.y * g.z;
              cnt += 1.f;
            }
          });
  if constexpr (kSolid) {
    float4* __restrict__ R = b.sgP + i;
    const size_t N = b.N;
    R[0] = make_float4(sg.x, sg.y, sg.z, cnt);
    R[N] = make_float4(p00, p11, p22, p01);
    R[2 * N] = make_float4(p02, p12, 0.f, 0.f);
  }
  const SVD s = svd3Fast(A);
  const float tol = 0.2f;
  V3 inv = splat(0.f);
  if (fabsf(s.sig.x) > tol) inv.x = __frcp_rn(s.sig.x);
  if (fabsf(s.sig.y) > tol) inv.y = __frcp_rn(s.sig.y);
  if (fabsf(s.sig.z) > tol) inv.z = __frcp_rn(s.sig.z);
  const M3 L = diagMul(s.V, inv, s.U);
  storeM(b.L, b.N, i, L);
  if constexpr (kVel) *out = SweepSums{Av, L, sg, p00, p11, p22, p01, p02, p12, cnt};
}
// The water particles' L of the last substep, from the same positions,
// neighbour lists and V^n as k_computeL would have used.
__global__ void XPBI_LB_COMPUTEL k_computeL_water(Bufs b) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  const float4 pi = b.posS[i];
  if (!waterW(pi.w)) return;
  bonetLok<false>(b, ctxOf(b, i), i, xyz(pi));
}

// The record solveB gathers from each solid neighbour, in four float4
// planes (plane f of slot i at Sp[f N + i]) so that one warp-wide gather of
// a field touches as few cache lines as the neighbour indices allow: dlam
// G L columns with the position in .w, then the position predicted with the
// velocities entering this iteration and the mass (the contact pass's
// inputs). The particle's own dv goes to SpSelf.
__device__ __forceinline__ void storeSp(const Bufs& b, uint32_t i, const M3& m, V3 self, V3 x, V3 xc, float mass) {
  float4* __restrict__ R = b.Sp + i;
  const size_t N = b.N;
  R[0] = make_float4(m.c[0].x, m.c[0].y, m.c[0].z, x.x);
  R[N] = make_float4(m.c[1].x, m.c[1].y, m.c[1].z, x.y);
  R[2 * N] = make_float4(m.c[2].x, m.c[2].y, m.c[2].z, x.z);
  R[3 * N] = make_float4(xc.x, xc.y, xc.z, mass);
  b.SpSelf[i] = make_float4(self.x, self.y, self.z, 0.f);
}

// Solid neighbours only: water entries are skipped before their data loads.
struct SolidOnly {
  __device__ __forceinline__ bool operator()(uint32_t e) const { return (e & kWaterBit) == 0u; }
};

// velocityGradient (simkernels.js:224-245) over the neighbour list.
__device__ __forceinline__ M3 velocityGradient(const Bufs& b, const Ctx& cx, uint32_t i, V3 xi, V3 vi,
                                               const float4* __restrict__ velIn) {
  const SceneDev& S = *cx.scene;
  const float4* __restrict__ posS = b.posS;
  // sum dv_b (L g_b)^T = (sum dv_b g_b^T) L^T: L applied once, after the loop
  M3 A = mzero();
  forNbrs(
      b, cx, i, xi, [&](uint32_t j) { return PV{ldg(posS + j), ldg(velIn + j)}; },
      [&](uint32_t, bool water, const PV& d) {
        if (water) return;
        const V3 g = gradWFast(S, xi - xyz(d.p));
        const V3 dv = (xyz(d.v) - vi) * d.v.w;
        A = madd(A, M3{{dv * g.x, dv * g.y, dv * g.z}});
      },
      SolidOnly{});
  return mul(A, transpose(loadM(b.L, b.N, i)));
}

// ---------------------------------------------------------------- solveA
// Inelastic constraint pass A (simkernels.js:248-309) in one neighbour sweep.
//
// The reference sweeps the neighbours twice: once for grad v (to form the
// trial F and the constraint gradient G L) and once for
//   denom = sum_b |g_b|^2 / m_b + |sgrad|^2 / m_i,  sgrad = -sum_b g_b,
//   cdot  = sum_b g_b . v_b + sgrad . v_i,           g_b = V_b (G L) gradW_b.
// With gt_b = L gradW_b (the term grad v already uses) and M = (dC/dF) F^nT,
// g_b = V_b M gt_b, so with the per-sweep sums
//   s = sum_b V_b gt_b,  Q = sum_b (V_b^2 / m_b) gt_b gt_b^T,  grad v = sum_b V_b (v_b - v_i) gt_b^T
// the second sweep reduces exactly to
//   sgrad = -M s,  denom = <M^T M, Q> + |sgrad|^2 / m_i,  cdot = <M, grad v>.
// (The last identity also removes the cancellation of the reference's
// sum_b g_b . v_b against sgrad . v_i when the body moves as a whole.)
// Constraint of a solid slot at the current velocities: the single sweep
// above plus the trial F, SVD, return map and the closed-form sums.
struct Constraint {
  float C;        // sqrt(2 Psi) at the projected state (0 below 1e-7)
  float denom;    // sum |grad C|^2 / m, self term included
  float cdot;     // grad C . v
  M3 GL;          // (dC/dF) F^nT L
  V3 sgrad;       // self gradient (per unit multiplier)
  V3 logSigTr;    // log of the trial singular values (clamped like safeSig)
  float nNbr;     // solid neighbours in the sweep
};

// (Compiled once, not inlined: solveA and computeL with features run the
// same instructions, so iteration 0's stored constraint is bit for bit the
// one solveA would evaluate; inlined, the compiler fuses multiplies and adds
// differently in each kernel.)
__device__ __noinline__ Constraint constraintFromSums(const SceneDev& S, const M3& A, V3 sg, float p00, float p11,
                                                     float p22, float p01, float p02, float p12, float cnt,
                                                     const M3& Li, const M3& Fn, const MatDev& m, float st);

template <int NL = 1>
__device__ __forceinline__ Constraint evalConstraint(const Bufs& b, const Ctx& cx, uint32_t i, float4 pi,
                                                     const float4* __restrict__ velIn, const MatDev& m, float st,
                                                     uint32_t lane = 0) {
  const SceneDev& S = *cx.scene;
  const float4* __restrict__ posS = b.posS;
  const V3 xi = xyz(pi);
  const V3 vi = xyz(velIn[i]);
  // The sums run over the raw kernel gradients g_b; the correction L is
  // applied once afterwards: with gt_b = L g_b,
  //   G = sum dv_b gt_b^T = A L^T,  s = L sum V_b g_b,  Q = L P L^T,
  // A = sum dv_b g_b^T, P = sum (V_b^2 / m_b) g_b g_b^T (same terms, the L
  // products factored out of the pair loop).
  M3 A = mzero();
  V3 sg = splat(0.f);
  float p00 = 0.f, p11 = 0.f, p22 = 0.f, p01 = 0.f, p02 = 0.f, p12 = 0.f, cnt = 0.f;
  if constexpr (NL == 1) {
    // s, P and the count do not depend on the velocities: computeL formed
    // them in the same order, so the sweep only accumulates A
    forNbrs(
        b, cx, i, xi, [&](uint32_t j) { return PV{ldg(posS + j), ldg(velIn + j)}; },
        [&](uint32_t, bool water, const PV& d) {
          if (water) return;
          addVelSum(A, d.v, vi, gradWFast(S, xi - xyz(d.p)));
        },
        SolidOnly{});
    const float4* __restrict__ R = b.sgP + i;
    const size_t N = b.N;
    const float4 r0 = R[0], r1 = R[N], r2 = R[2 * N];
    sg = xyz(r0);
    cnt = r0.w;
    p00 = r1.x;
    p11 = r1.y;
    p22 = r1.z;
    p01 = r1.w;
    p02 = r2.x;
    p12 = r2.y;
  } else {
    forNbrsLanes<NL>(
        b, cx, i, xi, lane, [&](uint32_t j) { return PV{ldg(posS + j), ldg(velIn + j)}; },
        [&](uint32_t, bool water, const PV& d) {
          if (water) return;
          const V3 g = gradWFast(S, xi - xyz(d.p));
          const float Vb = d.v.w;
          addVelSum(A, d.v, vi, g);
          sg = sg + g * Vb;
          const float c = Vb * Vb / cx.mats[matOfW(d.p.w)].mass;
          const V3 cg = g * c;
          p00 += cg.x * g.x;
          p11 += cg.y * g.y;
          p22 += cg.z * g.z;
          p01 += cg.x * g.y;
          p02 += cg.x * g.z;
          p12 += cg.y * g.z;
          cnt += 1.f;
        },
        SolidOnly{});
  }
  if constexpr (NL > 1) {
#pragma unroll
    for (int c = 0; c < 3; ++c) A.c[c] = laneSum<NL>(A.c[c]);
    sg = laneSum<NL>(sg);
    p00 = laneSum<NL>(p00);
    p11 = laneSum<NL>(p11);
    p22 = laneSum<NL>(p22);
    p01 = laneSum<NL>(p01);
    p02 = laneSum<NL>(p02);
    p12 = laneSum<NL>(p12);
    cnt = laneSum<NL>(cnt);
    if (lane != 0) return Constraint{};  // lane 0 finishes the slot
  }
  return constraintFromSums(S, A, sg, p00, p11, p22, p01, p02, p12, cnt, loadM(b.L, b.N, i), loadM(b.FS, b.N, i), m,
                            st);
}

// The per-particle part of the constraint from the sweep's sums (A = sum dv
// g^T, s = sum V g, P = sum (V^2/m) g g^T over the solid neighbours in list
// order, their count), the slot's correction L and its F.
__device__ __noinline__ Constraint constraintFromSums(const SceneDev& S, const M3& A, V3 sg, float p00, float p11,
                                                     float p22, float p01, float p02, float p12, float cnt,
                                                     const M3& Li, const M3& Fn, const MatDev& m, float st) {
  const M3 LiT = transpose(Li);
  const M3 G = mul(A, LiT);
  const V3 sv = mul(Li, sg);
  const M3 Qm = mul(mul(Li, M3{{v3(p00, p01, p02), v3(p01, p11, p12), v3(p02, p12, p22)}}), LiT);
  const float q00 = Qm.c[0].x, q11 = Qm.c[1].y, q22 = Qm.c[2].z;
  const float q01 = Qm.c[1].x, q02 = Qm.c[2].x, q12 = Qm.c[2].y;
  Constraint out;
  out.nNbr = cnt;
  const M3 Ftr = mul(madd(mident(), mscale(G, S.dt)), Fn);
  const SVD sd = svd3Fast(Ftr);
  out.logSigTr = vlog(safeSig(sd.sig));
  float stOut;
  const V3 sig = returnMap(sd.sig, m, st, S.dt, stOut);
  const float psi = stvkPsi(sig, m.mu, m.lam);
  out.C = sqrtf(fmaxf(2.f * psi, 0.f));
  if (out.C < 1e-7f) {
    out.C = 0.f;
    out.denom = 0.f;
    out.cdot = 0.f;
    out.GL = mzero();
    out.sgrad = splat(0.f);
    return out;
  }
  const V3 dpsi = stvkDPsi(sig, m.mu, m.lam);
  const M3 Pk = diagMul(sd.U, dpsi * __frcp_rn(out.C), sd.V);
  const M3 Mm = mul(Pk, transpose(Fn));
  out.GL = mul(Mm, Li);
  out.sgrad = -mul(Mm, sv);
  // <M^T M, Q> = sum over column pairs (a, b) of (M_a . M_b) Q_ab
  const V3 c0 = Mm.c[0], c1 = Mm.c[1], c2 = Mm.c[2];
  const float denomN = dot(c0, c0) * q00 + dot(c1, c1) * q11 + dot(c2, c2) * q22 +
                       2.f * (dot(c0, c1) * q01 + dot(c0, c2) * q02 + dot(c1, c2) * q12);
  out.denom = denomN + dot(out.sgrad, out.sgrad) / m.mass;
  out.cdot = dot(Mm.c[0], G.c[0]) + dot(Mm.c[1], G.c[1]) + dot(Mm.c[2], G.c[2]);
  return out;
}

// The iteration-0 constraint of slot i in four float4 planes (plane q of
// slot i at cons0[q N + i]): computeL with features evaluates it at the very
// velocities iteration 0 starts from, so iteration 0 can read it instead of
// sweeping the neighbours again.
__device__ __forceinline__ void storeConstraint(const Bufs& b, uint32_t i, const Constraint& c) {
  float4* __restrict__ R = b.cons0 + i;
  const size_t N = b.N;
  R[0] = make_float4(c.C, c.denom, c.cdot, c.sgrad.x);
  R[N] = make_float4(c.sgrad.y, c.sgrad.z, c.GL.c[0].x, c.GL.c[0].y);
  R[2 * N] = make_float4(c.GL.c[0].z, c.GL.c[1].x, c.GL.c[1].y, c.GL.c[1].z);
  R[3 * N] = make_float4(c.GL.c[2].x, c.GL.c[2].y, c.GL.c[2].z, 0.f);
}
__device__ __forceinline__ Constraint loadConstraint(const Bufs& b, uint32_t i) {
  const float4* __restrict__ R = b.cons0 + i;
  const size_t N = b.N;
  const float4 a = R[0], q = R[N], r = R[2 * N], t = R[3 * N];
  Constraint c;
  c.C = a.x;
  c.denom = a.y;
  c.cdot = a.z;
  c.sgrad = v3(a.w, q.x, q.y);
  c.GL = M3{{v3(q.z, q.w, r.x), v3(r.y, r.z, r.w), v3(t.x, t.y, t.z)}};
  return c;
}

__device__ __forceinline__ bool sceneDone(const Bufs& b, uint32_t i) {
  const uint32_t s = b.S > 1 ? (uint32_t)b.sceneOf[i] : 0u;
  return b.done[s] != 0;
}

// Whether slot i's scene iterates at iteration k: below its budget and not
// stopped, or in the plain re-solve (flags & kRerun) marked for it and below
// its own iteration count.
__device__ __forceinline__ bool iterating(const Bufs& b, const SceneDev& S, uint32_t i, int k, int flags) {
  const uint32_t s = b.S > 1 ? (uint32_t)b.sceneOf[i] : 0u;
  if (flags & kRerun) return b.rerun[s] != 0 && k < S.plainIterations;
  return k < S.iterations && b.done[s] == 0;
}

// Largest solid displacement dt |v| per scene entering iteration k (slot
// k & 1 of solidDisp, cleared by solveB(k - 1) or at the substep's start).
// Called by every thread of the warp before any of them leaves: the lanes of
// one scene combine their values and one of them raises the slot.
__device__ __forceinline__ void recordSolidDisp(const Bufs& b, uint32_t i, int k, float d) {
  const unsigned act = __activemask();
  const uint32_t sc = b.S > 1 ? (uint32_t)b.sceneOf[i] : 0u;
  const unsigned peers = b.S > 1 ? __match_any_sync(act, sc) : act;
  const unsigned mx = __reduce_max_sync(peers, __float_as_uint(d));  // d >= 0: bits order like values
  if ((threadIdx.x & 31u) == (unsigned)(__ffs(peers) - 1) && mx != 0u)
    atomicMax(b.solidDisp + (size_t)(k & 1) * b.S + sc, mx);
}

// ---------------------------------------------------------------- active set
// The learned solve's work skipping (flags kActive / kMarkMoved, never set by
// the reference solve). A slot's constraint depends on its own and its solid
// neighbours' velocities, its contact correction on the predicted positions
// of its solid neighbours: if none of those changed since the slot was last
// evaluated, its residuals are unchanged too. So from iteration 2 on
//   - solveA evaluates only the solids marked as changed (dirty); a solid
//     whose residual is within the scene's per-slot threshold takes no
//     impulse (its multiplier stays), the others update as the reference
//     does and mark their solid neighbours (bmark) for solveB;
//   - solveB visits only the changed or marked slots, updates velocities in
//     place (it reads no neighbour's velocity), applies a contact correction
//     only above the per-slot threshold, and a slot whose velocity changed
//     by more than the scene's velocity scale marks itself and its solid
//     neighbours as changed for the next iteration (as pbfB does);
//   - residuals of slots not visited keep their last values, so the scene's
//     residual sums and the early stop see every slot.
// Iterations 0 and 1 run every slot (iteration 0 moves every particle, so
// skipping in iteration 1 would find nothing to skip); iteration 1 starts
// the marking. The per-slot thresholds (formed once the
// iteration-0 sums are known) give each settled slot an equal share of
// asShare times the scene's residual budget, so settled slots alone can
// never hold the scene above its tolerance. The velocity scale is the same
// share of tol^2 times the mean squared velocity change of iteration 0: a
// change below it moves a neighbour's residual by about that neighbour's
// settle threshold or less, so the kept residuals are exact where nothing
// moved and otherwise off by at most that much (a tracked solve re-measures
// the final state over every slot).
__device__ __forceinline__ void countWarp(uint32_t* ctr) {
  const unsigned m = __activemask();
  if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) atomicAdd(ctr, (uint32_t)__popc(m));
}

// flag[j] = 1 for every solid neighbour j of slot i (list order; the stencil
// walk for an overflowed list). Plain byte stores: concurrent writers store
// the same value.
__device__ __forceinline__ void markSolidNbrs(const Bufs& b, const Ctx& cx, uint32_t i, V3 xi,
                                              uint8_t* __restrict__ flag) {
  const uint32_t cnt = b.nbrCount[i];
  if (cnt != kNbrOverflow) {
    const uint4* __restrict__ L = reinterpret_cast<const uint4*>(listOf(b.nbr, i));
    const uint32_t groups = (cnt + 3u) >> 2;
#pragma unroll 1
    for (uint32_t q = 0; q < groups; ++q) {
      const uint4 g = __ldg(L + q);
#pragma unroll
      for (uint32_t t = 0; t < 4u; ++t) {
        const uint32_t e = lane4(g, t);
        if (4u * q + t < cnt && !(e & kWaterBit)) flag[e] = 1;
      }
    }
  } else {
    const SceneDev& S = *cx.scene;
    forRows(S, b.cellStart, xi, [&](uint32_t beg, uint32_t end) {
#pragma unroll 1
      for (uint32_t j = beg; j < end; ++j) {
        if (j == i) continue;
        const float4 pj = ldg(b.posS + j);
        const V3 d = xi - xyz(pj);
        if (dot(d, d) < S.support2 && !waterW(pj.w)) flag[j] = 1;
      }
    });
  }
}

__device__ __forceinline__ uint32_t sceneIndex(const Bufs& b, const Ctx& cx) {
  return (uint32_t)(cx.scene - b.scenes);
}

// The iteration a launch works on: its argument, or inside the device loop
// (argument kIterDevice) the loop's current iteration.
__device__ __forceinline__ int iterK(const Bufs& b, int k) {
  return k == kIterDevice ? *reinterpret_cast<volatile const int*>(b.kIter) : k;
}

// Inelastic constraint pass A (simkernels.js:248-309).
//
// flags & kTrackResid: writes r^2 for the residual of the state entering
//   this iteration, r = C + alphaT lambda + gamma dt cdot (the numerator the
//   damped update drives to zero; without the damping term the Jacobi fixed
//   point sits at C + alphaT lambda = -gamma dt cdot, not 0), 0 for an
//   inactive constraint (C = 0), and at iteration 0 the residual at
//   lambda = 0 to c0sq. The tracked variant is a separate instantiation
//   (kTrack) so the plain path carries none of it.
// flags & kWarm (iteration 0): starts from lambda0 = lamWarm instead of 0.
//   Its impulse has not been applied to the velocities this pass sees, so the
//   first correction uses the linearised post-impulse residual: applying
//   lambda0 moves C by denom lambda0 and gamma dt cdot by gamma denom lambda0
//   (the particle's own response, the Jacobi diagonal), so
//     r = C + gamma dt cdot + ((1+gamma) denom + alphaT) lambda0,
//     dlam = -omega r / ((1+gamma) denom + alphaT),
//   and the applied impulse is lambda0 + dlam. A warm value that would not
//   reduce the particle's own residual, |r| >= |C + gamma dt cdot|, is
//   replaced by the plain start lambda0 = 0 (the plain solve stays the
//   fallback). With lambda0 = 0 both updates are the reference's.
// flags & kMeasureOnly: residual only (the pass after the last iteration).
// flags & kStoredC (iteration 0, after computeL with features, one lane per
//   slot): the constraint is the one computeL evaluated at the same
//   velocities; k_solveA_stored applies it without a neighbour sweep.
// G lanes per slot (G = 4 for small scenes): the lanes split the neighbour
// sweep, lane 0 finishes the slot.
//
// The update of slot i from its constraint c (lane 0 of the slot).
template <bool kTrack>
__device__ __forceinline__ void solveAUpdate(const Bufs& b, const Ctx& cx, uint32_t i, const float4& pi,
                                             const float4* __restrict__ velIn, uint32_t mi, const Constraint& c,
                                             int k, bool warm0, bool measure, bool act = false) {
  const SceneDev& S = *cx.scene;
  constexpr bool track = kTrack;
  const float g = S.kDamp;
  const float stiff = (1.f + g) * c.denom + S.alphaT;  // d(residual) / d(applied multiplier)
  const float r0 = c.C + g * S.dt * c.cdot;            // residual at lambda = 0
  float lam0 = k == 0 ? (warm0 ? b.lamWarm[i] : 0.f) : b.lam[i];
  if (warm0 && !(fabsf(r0 + stiff * lam0) < fabsf(r0))) lam0 = 0.f;
  // the quantity the update drives to zero: r = C + alphaT lambda + gamma dt cdot
  const float lamTerm = warm0 ? stiff * lam0 : S.alphaT * lam0;
  float r2 = 0.f;
  if (track) {
    // an inactive constraint (C below 1e-7: the reference skips the particle
    // and leaves its multiplier alone) has no residual; counting alphaT lambda
    // there would add a term no iteration can change
    const float r = c.C == 0.f ? 0.f : r0 + lamTerm;
    r2 = r * r;
    b.rr[i] = r2;
    if (k == 0) b.c0sq[i] = r0 * r0;
  }
  // an inactive constraint still takes part in the contact pass
  const V3 xi = xyz(pi);
  const V3 xci = xi + S.dt * xyz(velIn[i]);
  const float mass = cx.mats[mi].mass;
  if (measure) {  // the contact residual of these velocities, no impulse
    storeSp(b, i, mzero(), splat(0.f), xi, xci, mass);
    return;
  }
  if (kTrack && act && (c.C == 0.f || r2 <= b.thr[3 * sceneIndex(b, cx)])) {
    // settled (or inactive): no impulse (its stamp stays older than k + 1);
    // solveB reads only the predicted position and mass of such a slot
    b.Sp[3 * (size_t)b.N + i] = make_float4(xci.x, xci.y, xci.z, mass);
    return;
  }
  if (c.C == 0.f) {
    if (k == 0) b.lam[i] = lam0;
    storeSp(b, i, mzero(), splat(0.f), xi, xci, mass);
    return;
  }
  const float dlam = S.omega * (-c.C - lamTerm - g * S.dt * c.cdot) / stiff;
  b.lam[i] = lam0 + dlam;
  const float imp = warm0 ? lam0 + dlam : dlam;
  storeSp(b, i, mscale(c.GL, imp), c.sgrad * imp, xi, xci, mass);
  if (kTrack && act) {
    b.imp[i] = (uint8_t)(k + 1);
    // its residual moves with its multiplier even where the velocity change
    // rounds away: evaluate it again next iteration
    b.dirty[(k + 1) & 1][i] = 1;
    markSolidNbrs(b, cx, i, xi, b.bmark);  // their solveB applies this impulse
  }
}

template <bool kTrack, int kMinB, int G, int kBlock = kThreads>
__global__ void __launch_bounds__(kBlock, kMinB) k_solveA(Bufs b, int k, const float4* __restrict__ velIn,
                                                            int flags) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t / G, lane = t % G;
  if (i >= b.N) return;
  const Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  constexpr bool track = kTrack;
  const bool measure = kTrack && (flags & kMeasureOnly) != 0;  // measure passes are tracked ones
  const bool warm0 = (flags & kWarm) != 0 && k == 0;
  const float4 pi = b.posS[i];
  const bool active = measure || iterating(b, S, i, k, flags);
  // active set (one lane per slot): from iteration 2 a solid whose inputs
  // did not change keeps its residual and takes no impulse
  const bool act = kTrack && G == 1 && (flags & kActive) != 0 && k > 0;
  bool changed = true;
  if (act && active && !waterW(pi.w)) changed = b.dirty[k & 1][i] != 0;
  recordSolidDisp(b, i, k, active && !waterW(pi.w) && lane == 0 && changed ? S.dt * length(xyz(velIn[i])) : 0.f);
  if (!active || waterW(pi.w)) {  // water: its record is never read
    if (track && lane == 0) {
      b.rr[i] = 0.f;
      if (k == 0) b.c0sq[i] = 0.f;
    }
    return;
  }
  if (act) {
    if (!changed) return;
    countWarp(b.actA + k);
  }
  const uint32_t mi = matOfW(pi.w);
  const float st = b.stateS[i];
  const MatDev m = hardenedMat(cx.mats[mi], st);
  const Constraint c = evalConstraint<G>(b, cx, i, pi, velIn, m, st, lane);
  if (G > 1 && lane != 0) return;
  solveAUpdate<kTrack>(b, cx, i, pi, velIn, mi, c, k, warm0, measure, act);
}

// Active set, iterations from 2: the changed slots of the scenes still
// iterating, appended to a list (in no particular order: each slot's own
// sums keep their list order, so the results do not depend on it); which = 1
// lists the slots solveB updates (changed or receiving an impulse). Only
// solids are ever marked changed; k_solveA_list skips any water slot. The
// list's length is the iteration's visit count. Each thread reads the flags
// of 16 consecutive slots with one 16-byte load per array (the flag arrays
// are padded to a multiple of 16) and checks the few flagged ones; the
// block appends its slots with one atomic.
constexpr int kCompactSlots = 16;
constexpr int kCompactThreads = 256;
__global__ void __launch_bounds__(kCompactThreads) k_compact(Bufs b, int k, int which) {
  __shared__ uint32_t warpBase[kCompactThreads / 32];
  __shared__ uint32_t blockBase;
  k = iterK(b, k);
  const uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) * kCompactSlots;
  uint32_t take = 0;
  if (base < b.N) {
    uint4 f = *reinterpret_cast<const uint4*>(b.dirty[k & 1] + base);
    if (which == 1) {
      const uint4 m = *reinterpret_cast<const uint4*>(b.bmark + base);
      f.x |= m.x; f.y |= m.y; f.z |= m.z; f.w |= m.w;
    }
    const uint32_t w[4] = {f.x, f.y, f.z, f.w};
#pragma unroll
    for (int q = 0; q < kCompactSlots; ++q) {
      if (((w[q >> 2] >> (8 * (q & 3))) & 0xffu) == 0u) continue;
      const uint32_t i = base + (uint32_t)q;
      if (i >= b.N) break;
      const uint32_t s = b.S > 1 ? (uint32_t)b.sceneOf[i] : 0u;
      if (k < b.scenes[s].iterations && !b.done[s]) take |= 1u << q;
    }
  }
  const uint32_t cnt = (uint32_t)__popc(take);
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t incl = cnt;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t n = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= (unsigned)off) incl += n;
  }
  if (lane == 31u) warpBase[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
#pragma unroll
    for (int q = 0; q < kCompactThreads / 32; ++q) {
      const uint32_t t = warpBase[q];
      warpBase[q] = run;
      run += t;
    }
    blockBase = run ? atomicAdd(which == 0 ? b.actA + k : b.actB + k, run) : 0u;
  }
  __syncthreads();
  if (!take) return;
  uint32_t start = blockBase + warpBase[warp] + incl - cnt;
  uint32_t* out = which == 0 ? b.listA : b.listB;
  while (take) {
    const int q = __ffs(take) - 1;
    take &= take - 1u;
    out[start++] = base + (uint32_t)q;
  }
}

// solveA over listA (iterations k >= 1 of the active set): the listed slots
// with a grid-stride loop over a grid that fills the GPU once, so warps stay
// full however the listed slots are spread.
template <int kMinB, int kBlock>
__global__ void __launch_bounds__(kBlock, kMinB) k_solveA_list(Bufs b, int k, const float4* __restrict__ velIn,
                                                                int flags) {
  k = iterK(b, k);
  const uint32_t cnt = *(volatile const uint32_t*)(b.actA + k);
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < cnt; t += gridDim.x * blockDim.x) {
    const uint32_t i = b.listA[t];
    const float4 pi = b.posS[i];
    if (waterW(pi.w)) continue;  // water takes no constraint (none is ever marked)
    const Ctx cx = ctxOf(b, i);
    const SceneDev& S = *cx.scene;
    recordSolidDisp(b, i, k, S.dt * length(xyz(velIn[i])));
    const uint32_t mi = matOfW(pi.w);
    const float st = b.stateS[i];
    const MatDev m = hardenedMat(cx.mats[mi], st);
    const Constraint c = evalConstraint<1>(b, cx, i, pi, velIn, m, st, 0);
    solveAUpdate<true>(b, cx, i, pi, velIn, mi, c, k, false, false, true);
  }
  (void)flags;
}

// Iteration 0 after computeL with features: the constraint it stored at
// these velocities (bit-identical to evaluating it), no neighbour sweep — a
// register-light launch at full occupancy in place of the sweep kernel.
template <bool kTrack>
__global__ void __launch_bounds__(kThreads) k_solveA_stored(Bufs b, const float4* __restrict__ velIn, int flags) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  const Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  const bool warm0 = (flags & kWarm) != 0;
  const float4 pi = b.posS[i];
  const bool active = 0 < S.iterations && !sceneDone(b, i);
  recordSolidDisp(b, i, 0, active && !waterW(pi.w) ? S.dt * length(xyz(velIn[i])) : 0.f);
  if (!active || waterW(pi.w)) {
    if (kTrack) {
      b.rr[i] = 0.f;
      b.c0sq[i] = 0.f;
    }
    return;
  }
  solveAUpdate<kTrack>(b, cx, i, pi, velIn, matOfW(pi.w), loadConstraint(b, i), 0, warm0, false);
}

// Network features of every slot at iteration 0 (zeros for water):
//   0-2  log singular values of the trial F
//   3    C = sqrt(2 Psi) at the projected trial state
//   4    alphaT * lambda of the previous substep (same particle)
//   5    alphaT * lambda_1, lambda_1 = -C / (denom + alphaT): the particle's
//        own Newton step, blind to its neighbours
//   6    log10(1 + denom / alphaT): stiffness of the constraint vs compliance
//   7    solid neighbours / 32
//   8-14 material kind one-hot
//   15   log10(mu) - 4.5
__device__ __forceinline__ void fillFeatures(float (&f)[kFeat], const SceneDev& S, const Constraint& c, float lamPrev,
                                             uint32_t kind, const MatDev& m) {
  const float aT = S.alphaT;
  f[0] = c.logSigTr.x;
  f[1] = c.logSigTr.y;
  f[2] = c.logSigTr.z;
  f[3] = c.C;
  f[4] = aT * lamPrev;
  f[5] = -c.C * aT / (c.denom + aT);
  f[6] = log10f(1.f + c.denom / aT);
  f[7] = c.nNbr * (1.f / 32.f);
#pragma unroll
  for (uint32_t q = 0; q < 7u; ++q) f[8 + q] = kind == q ? 1.f : 0.f;  // constant indices: f stays in registers
  f[15] = log10f(fmaxf(m.mu, 1e-6f)) - 4.5f;
}
__device__ __forceinline__ void storeFeatures(const Bufs& b, uint32_t i, const float (&f)[kFeat]) {
  float4* out = reinterpret_cast<float4*>(b.feat + (size_t)i * kFeat);
#pragma unroll
  for (int q = 0; q < kFeat / 4; ++q) out[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
}

// Bonet-Lok correction with SVD pseudo-inverse (simkernels.js:189-221); its
// candidate walk records the substep's neighbour list. kFeatures (the
// learned solve, or features logged): the same sweep forms iteration 0's
// velocity sum, so iteration 0's constraint (the arithmetic solveA's sweep
// would do, from the same sums in the same order) is stored for
// k_solveA_stored here, with the network's features (fillFeatures; zeros
// for water and for scenes without iterations), without a second sweep of
// every solid's neighbours.
template <bool kSums, bool kFeatures>
__device__ __forceinline__ void computeL(const Bufs& b) {
  static_assert(kSums || !kFeatures, "the features need the sums");
  // blocks run last to first: the pass starts where the reorder ended, on
  // slots whose data is still in L2
  const uint32_t i = (gridDim.x - 1u - blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  const Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  const float4* __restrict__ posS = b.posS;
  const float4 pi = posS[i];
  const V3 xi = xyz(pi);
  const float s2 = S.support2;
  const uint32_t cnt = recordCandidates(S, b.cellStart, xi, i, listOf(b.nbr, i), [&](uint32_t j, uint32_t& e) {
    const float4 p = ldg(posS + j);
    const V3 d = xi - xyz(p);
    e = j | (__float_as_uint(p.w) & kWaterBit);  // the water flag is the sign bit of pos.w
    return dot(d, d) < s2;
  });
  b.nbrCount[i] = cnt <= kNbrCap ? cnt : kNbrOverflow;
  // no pass of the substep reads a water particle's correction (every
  // velocity gradient is a solid's): k_computeL_water forms it when the state
  // is read
  if constexpr (kFeatures) {
    float f[kFeat];
#pragma unroll
    for (int q = 0; q < kFeat; ++q) f[q] = 0.f;
    if (!waterW(pi.w)) {
      SweepSums w;
      bonetLok<true, true>(b, cx, i, xi, &w);
      if (S.iterations > 0) {
        const uint32_t mi = matOfW(pi.w);
        const float st = b.stateS[i];
        const MatDev m = hardenedMat(cx.mats[mi], st);
        const Constraint c = constraintFromSums(S, w.Av, w.sg, w.p00, w.p11, w.p22, w.p01, w.p02, w.p12, w.cnt, w.L,
                                                loadM(b.FS, b.N, i), m, st);
        storeConstraint(b, i, c);
        fillFeatures(f, S, c, b.lamPrev[i], cx.mats[mi].kind, m);
      }
    }
    storeFeatures(b, i, f);
  } else {
    if (!waterW(pi.w)) bonetLok<kSums>(b, cx, i, xi);
  }
}
template <bool kSums>
__global__ void XPBI_LB_COMPUTEL k_computeL(Bufs b) {
  computeL<kSums, false>(b);
}
__global__ void XPBI_LB_COMPUTEL_FEATURES k_computeL_features(Bufs b) { computeL<true, true>(b); }

// lambda_warm = previous multiplier + network output / alphaT (the network
// predicts alphaT times the increment over the previous substep's multiplier)
__global__ void k_warm_from_net(Bufs b) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  const Ctx cx = ctxOf(b, i);
  const float4 pi = b.posS[i];
  b.lamWarm[i] = waterW(pi.w) ? 0.f : b.lamPrev[i] + b.netOut[i] / cx.scene->alphaT;
}

// warm start from the previous substep's multiplier alone (no network)
__global__ void k_warm_from_prev(Bufs b) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  b.lamWarm[i] = b.lamPrev[i];
}

// Per-scene residual norms, deterministic, in one launch: block (x, s)
// sums the x-th of the scene's residBlocks(n) consecutive slot ranges (at
// least kResidPerBlock slots each, at most kResidBlocks ranges, so a large
// scene fills the GPU with float4 loads in flight and a small one takes few
// blocks) in a fixed order and stores the range's partial sums; the last of
// the scene's blocks to finish (a ticket counter, no waiting) adds the
// partials in range order, so the totals do not depend on which block comes
// last.
// Sums: constraint residual^2, (iteration 0) residual^2 at lambda = 0,
// contact correction^2, (iteration 0) velocity change^2.
// Each thread sums in f32 in a fixed order (a convergence test on sums of
// squares needs nothing finer, and f64 is slow here), then a fixed warp
// butterfly; the warps of a block and the ranges of a scene are added in f64.
//
// k >= 0: the residuals of the state entering iteration k (early stop),
// reduced after iteration k's update; k < 0: after the last iteration (slot
// kMaxResid - 1). A scene stops, skipping iterations k+1.., once both its
// constraint residual and its contact residual are within tol of their
// values entering iteration 0 (an early stop also ends the contact passes,
// which the constraint residual does not see). With a warm start, iteration
// 0's constraint residual is the linearised estimate before the warm impulse
// is applied, so it never stops the solve.
constexpr int kResidSums = 4;
constexpr int kResidThreads = 256;
constexpr uint32_t kResidPerBlock = 4096;
static_assert(kResidBlocks % 32 == 0, "whole lanes of partials in the final sum");
__host__ __device__ __forceinline__ uint32_t residBlocks(uint32_t n) {
  const uint32_t g = (n + kResidPerBlock - 1u) / kResidPerBlock;
  return g < 1u ? 1u : (g > (uint32_t)kResidBlocks ? (uint32_t)kResidBlocks : g);
}
__global__ void __launch_bounds__(kResidThreads) k_resid(Bufs b, int k, int warm) {
  __shared__ float warpSum[kResidThreads / 32][kResidSums];
  __shared__ bool lastBlock;
  k = iterK(b, k);
  const uint32_t s = blockIdx.y;
  const SceneDev& S = b.scenes[s];
  const uint32_t n = S.n, base = S.pBase;
  const uint32_t G = residBlocks(n);
  if (blockIdx.x >= G) return;  // the whole block: this scene needs fewer ranges
  const uint32_t c = blockIdx.x;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t lo = base + (uint32_t)(((uint64_t)n * c) / G);
  const uint32_t hi = base + (uint32_t)(((uint64_t)n * (c + 1)) / G);
  float a = 0.f, a0 = 0.f, ac = 0.f, av = 0.f;
  const bool velSum = k == 0 && S.asShare > 0.f;  // the active set's velocity-change scale
  if (!b.done[s] || k < 0) {
    // the range's 16-byte-aligned interior as float4 (the arrays start on
    // 256-byte boundaries), its ragged ends (< 4 slots each) as scalars
    const uint32_t lo4 = min(hi, (lo + 3u) & ~3u), hi4 = max(lo4, hi & ~3u);
    if (lo + tid < lo4) {
      a += b.rr[lo + tid];
      ac += b.rc[lo + tid];
      if (k == 0) a0 += b.c0sq[lo + tid];
      if (velSum) av += b.dv0sq[lo + tid];
    }
    if (hi4 + tid < hi) {
      a += b.rr[hi4 + tid];
      ac += b.rc[hi4 + tid];
      if (k == 0) a0 += b.c0sq[hi4 + tid];
      if (velSum) av += b.dv0sq[hi4 + tid];
    }
    const float4* __restrict__ rr4 = reinterpret_cast<const float4*>(b.rr);
    const float4* __restrict__ rc4 = reinterpret_cast<const float4*>(b.rc);
    const float4* __restrict__ c04 = reinterpret_cast<const float4*>(b.c0sq);
#pragma unroll 4
    for (uint32_t q = lo4 / 4u + tid; q < hi4 / 4u; q += kResidThreads) {
      const float4 x = rr4[q], y = rc4[q];
      a += (x.x + x.y) + (x.z + x.w);
      ac += (y.x + y.y) + (y.z + y.w);
      if (k == 0) {
        const float4 z = c04[q];
        a0 += (z.x + z.y) + (z.z + z.w);
      }
      if (velSum) {
        const float4 z = reinterpret_cast<const float4*>(b.dv0sq)[q];
        av += (z.x + z.y) + (z.z + z.w);
      }
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, off);
    a0 += __shfl_xor_sync(0xffffffffu, a0, off);
    ac += __shfl_xor_sync(0xffffffffu, ac, off);
    av += __shfl_xor_sync(0xffffffffu, av, off);
  }
  if (lane == 0) {
    warpSum[warp][0] = a;
    warpSum[warp][1] = a0;
    warpSum[warp][2] = ac;
    warpSum[warp][3] = av;
  }
  __syncthreads();
  if (tid == 0) {
    double t[kResidSums] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int w = 0; w < kResidThreads / 32; ++w)
#pragma unroll
      for (int q = 0; q < kResidSums; ++q) t[q] += (double)warpSum[w][q];
    double* part = b.residPart + ((size_t)s * kResidBlocks + c) * kResidSums;
#pragma unroll
    for (int q = 0; q < kResidSums; ++q) part[q] = t[q];
    __threadfence();  // the partials are visible before this block's ticket
    lastBlock = atomicAdd(b.residTicket + s, 1u) == G - 1u;
  }
  __syncthreads();
  if (!lastBlock || tid >= 32u) return;
  // the scene's last block, one warp: lane l adds ranges l, l + 32, ... in
  // order (loads through L2: the other blocks' partials are not in this
  // SM's L1), then a fixed butterfly combines the lanes
  __threadfence();
  if (lane == 0) b.residTicket[s] = 0u;  // every block of this launch has taken its ticket
  if (k >= 0 && (b.done[s] || k >= S.iterations)) return;
  double ta = 0.0, ta0 = 0.0, tac = 0.0, tav = 0.0;
#pragma unroll
  for (int r = 0; r < kResidBlocks / 32; ++r) {
    const uint32_t q = lane + 32u * (uint32_t)r;
    if (q < G) {
      const double* part = b.residPart + ((size_t)s * kResidBlocks + q) * kResidSums;
      ta += __ldcg(part);
      ta0 += __ldcg(part + 1);
      tac += __ldcg(part + 2);
      tav += __ldcg(part + 3);
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    ta += __shfl_xor_sync(0xffffffffu, ta, off);
    ta0 += __shfl_xor_sync(0xffffffffu, ta0, off);
    tac += __shfl_xor_sync(0xffffffffu, tac, off);
    tav += __shfl_xor_sync(0xffffffffu, tav, off);
  }
  if (lane != 0) return;
  if (k < 0) {
    b.resid[(size_t)s * kMaxResid + (kMaxResid - 1)] = ta;
    b.residC[(size_t)s * kMaxResid + (kMaxResid - 1)] = tac;
    return;
  }
  if (k < kMaxResid - 1) {
    b.resid[(size_t)s * kMaxResid + k] = ta;
    b.residC[(size_t)s * kMaxResid + k] = tac;
  }
  const double tol = (double)S.residTol, tolC = (double)S.residTolC;
  if (k == 0) {
    b.c0[s] = ta0;
    b.cc0[s] = tac;
    // active set: a settled slot may hold up to asShare / nSolid of the
    // scene's squared residual budget (tol^2 of the iteration-0 sums)
    const double share = (double)S.asShare / (double)max(S.nSolid, 1u);
    b.thr[3 * s] = (float)(share * tol * tol * ta0);
    b.thr[3 * s + 1] = (float)(share * tolC * tolC * tac);
    // a velocity change at the scale the converged solve still makes (the
    // tolerance times iteration 0's) moves a neighbour's residual by about
    // its own settle threshold: smaller ones do not count as moved
    b.thr[3 * s + 2] = (float)(share * tol * tol * tav);
  }
  if (tol > 0.0 && ta <= tol * tol * b.c0[s] && tac <= tolC * tolC * b.cc0[s] && !(warm && k == 0)) b.done[s] = 1;
  b.itersUsed[s] = k + 1;
}

// keep this substep's final multipliers for the next substep's features
__global__ void k_keep_lambda(Bufs b) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  b.lamOut[i] = b.lam[i];
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

struct SBData {
  float4 r0, r1, r2;  // a neighbour's dlam G L columns with its position in .w (the record's first planes)
};

// ---------------------------------------------------------------- solveB
// Constraint dv gather + contact correction + boundaries (simkernels.js:315-366).
// When a PBF pass follows, also stores the predicted position x + dt v_out
// that pbfA / pbfB would otherwise recompute for every candidate.
// flags & kTrackResid: writes |contact correction|^2 of the velocities
//   entering this iteration to rc (the contact residual; 0 for water).
// flags & kMeasureOnly: the contact residual only, of every solid slot, no
//   velocity update (the pass after the last iteration).
template <int kMinB, int G, int kBlock = kThreads>
__global__ void __launch_bounds__(kBlock, kMinB) k_solveB(Bufs b, int k, const float4* __restrict__ velIn,
                                                      float4* __restrict__ velOut, int writeXc, int flags) {
  // blocks run last to first: the pass starts where solveA ended, on slots
  // whose data is still in L2
  const uint32_t t = (gridDim.x - 1u - blockIdx.x) * blockDim.x + threadIdx.x;
  const uint32_t i = t / G, lane = t % G;
  for (uint32_t q = t; q < b.S; q += gridDim.x * blockDim.x)  // the next iteration's slot
    b.solidDisp[(size_t)((k + 1) & 1) * b.S + q] = 0u;
  if (i >= b.N) return;
  const Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  const float4* __restrict__ posS = b.posS;
  const float4* __restrict__ Sp = b.Sp;
  const float4 vi4 = velIn[i];
  const float4 pi = posS[i];
  const bool track = (flags & kTrackResid) != 0;
  const bool measure = (flags & kMeasureOnly) != 0;
  if (!measure && !iterating(b, S, i, k, flags)) {
    if (lane == 0) {
      velOut[i] = vi4;
      if (writeXc) {
        const V3 xc = xyz(pi) + S.dt * xyz(vi4);
        b.xc[i] = make_float4(xc.x, xc.y, xc.z, pi.w);
      }
    }
    return;
  }
  const uint32_t mi = matOfW(pi.w);
  const MatDev& m = cx.mats[mi];
  const V3 xi = xyz(pi);
  V3 dv = splat(0.f), corr = splat(0.f);
  if (!waterW(pi.w)) {
    const size_t N = b.N;
    if (G == 1) dv = xyz(b.SpSelf[i]);
    const float Vi = vi4.w;
    const V3 xci = xi + S.dt * xyz(vi4);
    const float minD = S.minD;
    const float massI = m.mass;
    // A neighbour can be within minD of x_i + dt v_i at the predicted
    // positions only if |x_b - x_i| < minD + dt |v_i| + dt |v_b|, and dt |v_b|
    // is at most the scene's largest solid displacement this iteration
    // (recorded by solveA): farther neighbours skip the contact test and the
    // load of their predicted position. 1% of slack covers the rounding of
    // the predicted positions and of the bound; the test on the pairs that
    // remain is unchanged, so the result is too.
    const float reach = (minD + S.dt * length(xyz(vi4)) +
                         __uint_as_float(__ldg(b.solidDisp + (size_t)(k & 1) * b.S + (cx.scene - b.scenes)))) *
                        1.01f;
    const float reach2 = reach * reach;
    auto body = [&](uint32_t j, bool water, const SBData& d) {
      if (water) return;
      const V3 pb = v3(d.r0.w, d.r1.w, d.r2.w);
      const M3 Sb = {{xyz(d.r0), xyz(d.r1), xyz(d.r2)}};
      const V3 dxp = pb - xi;
      dv = dv + Vi * mul(Sb, gradWFast(S, dxp));
      if (!(dot(dxp, dxp) < reach2)) return;
      const float4 r3 = ldg(Sp + 3 * b.N + j);
      const V3 dxc = xci - xyz(r3);
      const float d2 = dot(dxc, dxc);
      if (d2 < minD * minD && d2 > 1e-18f) {
        const float rinv = rsqrtf(d2);
        const float dist = d2 * rinv;
        const float mb = r3.w;
        const float w = mb / (massI + mb);
        corr = corr + dxc * (rinv * ((minD - dist) * w));
      }
    };
    const uint32_t cnt = b.nbrCount[i];
    if (G > 1 && cnt != kNbrOverflow) {
      // lane `lane` takes the entries k % G == lane, skipping water ones
      const uint4* __restrict__ L = reinterpret_cast<const uint4*>(listOf(b.nbr, i));
      const uint32_t groups = (cnt + 3u) >> 2;
#pragma unroll 1
      for (uint32_t q = 0; q < groups; ++q) {
        const uint4 grp = __ldg(L + q);
#pragma unroll
        for (uint32_t s = lane; s < 4u; s += G) {
          const uint32_t e = lane4(grp, s);
          if (4u * q + s < cnt && !(e & kWaterBit)) {
            const float4* R = Sp + e;
            body(e, false, SBData{ldg(R), ldg(R + N), ldg(R + 2 * N)});
          }
        }
      }
    } else if (G == 1 && cnt != kNbrOverflow) {
      // water neighbours are skipped before their record is loaded
      forList<true>(listOf(b.nbr, i), cnt,
                    [&](uint32_t e) {
                      SBData d;
                      if (e & kWaterBit) {
                        d.r0 = d.r1 = d.r2 = make_float4(0.f, 0.f, 0.f, 0.f);
                      } else {
                        const float4* R = Sp + e;
                        d.r0 = ldg(R);
                        d.r1 = ldg(R + N);
                        d.r2 = ldg(R + 2 * N);
                      }
                      return d;
                    },
                    [&](uint32_t j, bool water, const SBData& d) { body(j, water, d); });
    } else {
      forRows(S, b.cellStart, xi, [&](uint32_t beg, uint32_t end) {
#pragma unroll 1
        for (uint32_t j = beg + lane; j < end; j += G) {
          if (j == i) continue;
          const float4 pj = ldg(posS + j);
          const V3 d = xi - xyz(pj);
          if (dot(d, d) < S.support2 && !waterW(pj.w)) {
            const float4* R = Sp + j;
            body(j, false, SBData{ldg(R), ldg(R + N), ldg(R + 2 * N)});
          }
        }
      });
    }
    if constexpr (G > 1) {
      dv = laneSum<G>(dv) + xyz(b.SpSelf[i]);
      corr = laneSum<G>(corr);
    }
  }
  if (G > 1 && lane != 0) return;
  if (track) b.rc[i] = dot(corr, corr);
  if (measure) return;
  V3 dvv = dv / (m.mass * S.dt);
  const float dvl = length(dvv);
  if (dvl > S.dvCap) dvv = dvv * (S.dvCap / dvl);
  V3 v = xyz(vi4) + dvv + corr * (S.contactOmega / S.dt);
  v = applyBoundary(S, xi + S.dt * v, v, xi, m.boundFriction);
  velOut[i] = make_float4(v.x, v.y, v.z, vi4.w);
  if (writeXc) {
    const V3 xc = xi + S.dt * v;
    b.xc[i] = make_float4(xc.x, xc.y, xc.z, pi.w);
  }
}

// solveB under the active set (one lane per slot; the launch passes
// velOut == velIn: a slot reads only its own velocity, so the update is in
// place and slots not visited keep theirs without a copy). flags & kActive
// (iterations >= 2): only slots marked as changed (dirty) or receiving a
// neighbour's impulse (bmark) run; a changed slot re-evaluates its contact
// correction and applies it only above the scene's per-slot threshold, a
// slot that only receives impulses keeps its (unchanged, unapplied)
// contact correction. A neighbour's impulse record is gathered only if it
// took an impulse (imp); its predicted position and mass (the record's
// fourth plane) are current for every solid. flags & kMarkMoved: a slot
// whose velocity changed marks itself and its solid neighbours as changed
// for iteration k + 1. The scene's solid displacement bound carries into
// the next iteration's slot (solveA raises it for the slots it visits).
// One slot of solveB under the active set; `listed`: the slot came from
// listB (changed or marked), so the flags are only cleared.
__device__ __forceinline__ void solveBActiveSlot(const Bufs& b, int k, float4* __restrict__ vel, int writeXc,
                                                 int flags, uint32_t i, bool listed) {
  const Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  const float4 pi = b.posS[i];
  if (k >= S.iterations || sceneDone(b, i)) {
    if (writeXc) {
      const float4 vi4 = vel[i];
      const V3 xc = xyz(pi) + S.dt * xyz(vi4);
      b.xc[i] = make_float4(xc.x, xc.y, xc.z, pi.w);
    }
    return;
  }
  // water: solveB only applies the boundary to it, which after iteration 0
  // the PBF pass that moved it has already done (pbfB folds it in)
  if (k > 0 && waterW(pi.w)) {
    if (writeXc) {
      const float4 vi4 = vel[i];
      const V3 xc = xyz(pi) + S.dt * xyz(vi4);
      b.xc[i] = make_float4(xc.x, xc.y, xc.z, pi.w);
    }
    return;
  }
  const bool skip = (flags & kActive) != 0 && k > 0;
  bool changed = true;
  if (skip) {
    uint8_t* __restrict__ dk = b.dirty[k & 1];
    changed = dk[i] != 0;
    const bool marked = b.bmark[i] != 0;
    if (changed) dk[i] = 0;
    if (marked) b.bmark[i] = 0;
    if (!changed && !marked) {
      if (writeXc) {
        const float4 vi4 = vel[i];
        const V3 xc = xyz(pi) + S.dt * xyz(vi4);
        b.xc[i] = make_float4(xc.x, xc.y, xc.z, pi.w);
      }
      return;
    }
    if (!listed) countWarp(b.actB + k);
  }
  const uint8_t stamp = (uint8_t)(k + 1);
  const float4 vi4 = vel[i];
  const uint32_t mi = matOfW(pi.w);
  const MatDev& m = cx.mats[mi];
  const V3 xi = xyz(pi);
  const bool iWater = waterW(pi.w);
  V3 dv = splat(0.f), corr = splat(0.f);
  if (!iWater) {
    const size_t N = b.N;
    const float4* __restrict__ Sp = b.Sp;
    if (!skip || b.imp[i] == stamp) dv = xyz(b.SpSelf[i]);
    const float Vi = vi4.w;
    const V3 xci = xi + S.dt * xyz(vi4);
    const float minD = S.minD;
    const float massI = m.mass;
    const float reach = (minD + S.dt * length(xyz(vi4)) +
                         __uint_as_float(__ldg(b.solidDisp + (size_t)(k & 1) * b.S + sceneIndex(b, cx)))) *
                        1.01f;
    const float reach2 = reach * reach;
    auto contact = [&](const float4& r3) {
      const V3 dxc = xci - xyz(r3);
      const float d2 = dot(dxc, dxc);
      if (d2 < minD * minD && d2 > 1e-18f) {
        const float rinv = rsqrtf(d2);
        const float dist = d2 * rinv;
        const float mb = r3.w;
        const float w = mb / (massI + mb);
        corr = corr + dxc * (rinv * ((minD - dist) * w));
      }
    };
    auto visit = [&](uint32_t j) {
      const bool jImp = !skip || b.imp[j] == stamp;
      if (jImp) {
        const float4* R = Sp + j;
        const float4 r0 = ldg(R), r1 = ldg(R + N), r2 = ldg(R + 2 * N);
        const V3 pb = v3(r0.w, r1.w, r2.w);
        const M3 Sb = {{xyz(r0), xyz(r1), xyz(r2)}};
        const V3 dxp = pb - xi;
        dv = dv + Vi * mul(Sb, gradWFast(S, dxp));
        if (changed && dot(dxp, dxp) < reach2) contact(ldg(Sp + 3 * N + j));
      } else if (changed) {
        contact(ldg(Sp + 3 * N + j));
      }
    };
    const uint32_t cnt = b.nbrCount[i];
    if (cnt != kNbrOverflow) {
      const uint4* __restrict__ L = reinterpret_cast<const uint4*>(listOf(b.nbr, i));
      const uint32_t groups = (cnt + 3u) >> 2;
#pragma unroll 1
      for (uint32_t q = 0; q < groups; ++q) {
        const uint4 g = __ldg(L + q);
#pragma unroll
        for (uint32_t t = 0; t < 4u; ++t) {
          const uint32_t e = lane4(g, t);
          if (4u * q + t < cnt && !(e & kWaterBit)) visit(e);
        }
      }
    } else {
      forRows(S, b.cellStart, xi, [&](uint32_t beg, uint32_t end) {
#pragma unroll 1
        for (uint32_t j = beg; j < end; ++j) {
          if (j == i) continue;
          const float4 pj = ldg(b.posS + j);
          const V3 d = xi - xyz(pj);
          if (dot(d, d) < S.support2 && !waterW(pj.w)) visit(j);
        }
      });
    }
    if (changed) {
      const float c2 = dot(corr, corr);
      b.rc[i] = c2;
      if (skip && c2 <= b.thr[3 * sceneIndex(b, cx) + 1]) corr = splat(0.f);  // settled: left unapplied
    } else {
      corr = splat(0.f);  // unchanged since last evaluated: at or below the threshold, not applied
    }
  } else if (changed) {
    b.rc[i] = 0.f;
  }
  V3 dvv = dv / (m.mass * S.dt);
  const float dvl = length(dvv);
  if (dvl > S.dvCap) dvv = dvv * (S.dvCap / dvl);
  V3 v = xyz(vi4) + dvv + corr * (S.contactOmega / S.dt);
  v = applyBoundary(S, xi + S.dt * v, v, xi, m.boundFriction);
  vel[i] = make_float4(v.x, v.y, v.z, vi4.w);
  if (writeXc) {
    const V3 xc = xi + S.dt * v;
    b.xc[i] = make_float4(xc.x, xc.y, xc.z, pi.w);
  }
  const V3 dvel = v - xyz(vi4);
  const float dv2 = dot(dvel, dvel);
  if (k == 0) b.dv0sq[i] = iWater ? 0.f : dv2;
  // moved: any change in iteration 0; later, a change above the scene's scale
  if ((flags & kMarkMoved) && (k == 0 ? (v.x != vi4.x || v.y != vi4.y || v.z != vi4.z)
                                      : dv2 > b.thr[3 * sceneIndex(b, cx) + 2])) {
    uint8_t* __restrict__ dn = b.dirty[(k + 1) & 1];
    dn[i] = 1;
    if (!iWater) markSolidNbrs(b, cx, i, xi, dn);
  }
}

// solveB under the active set (one lane per slot; the launch passes one
// velocity array: a slot reads only its own velocity, so the update is in
// place and slots not visited keep theirs without a copy). flags & kActive
// (iterations >= 2): only slots marked as changed (dirty) or receiving a
// neighbour's impulse (bmark) run; a changed slot re-evaluates its contact
// correction and applies it only above the scene's per-slot threshold, a
// slot that only receives impulses keeps its (unchanged, unapplied)
// contact correction. A neighbour's impulse record is gathered only if it
// took an impulse this iteration (its stamp is k + 1); its predicted
// position and mass (the record's fourth plane) are current for every
// solid. flags & kMarkMoved: a slot whose velocity changed (after iteration
// 0: by more than the scene's velocity scale) marks itself and its solid
// neighbours as changed for iteration k + 1. The scene's solid displacement
// bound carries into the next iteration's slot (solveA raises it for the
// slots it visits). With `list` the launch runs over listB (grid-stride),
// else one thread per slot.
template <int kMinB, int kBlock = kThreads>
__global__ void __launch_bounds__(kBlock, kMinB) k_solveB_active(Bufs b, int k, float4* __restrict__ vel, int writeXc,
                                                                 int flags, int list) {
  k = iterK(b, k);
  const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
  for (uint32_t q = t0; q < b.S; q += gridDim.x * blockDim.x)  // carried into the next iteration's slot
    b.solidDisp[(size_t)((k + 1) & 1) * b.S + q] = b.solidDisp[(size_t)(k & 1) * b.S + q];
  if (list) {
    const uint32_t cnt = *(volatile const uint32_t*)(b.actB + k);
    for (uint32_t t = t0; t < cnt; t += gridDim.x * blockDim.x)
      solveBActiveSlot(b, k, vel, writeXc, flags, b.listB[t], true);
    return;
  }
  const uint32_t i = (gridDim.x - 1u - blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < b.N) solveBActiveSlot(b, k, vel, writeXc, flags, i, false);
}

__device__ __forceinline__ bool pbfActive(const SceneDev& S, int k) {
  return S.hasWater && k < S.pbfUntil;
}

// ---------------------------------------------------------------- pbfA
// PBF density multiplier (simkernels.js:407-439). Walks the stencil around
// the current cell with predicted positions and records, in order, the
// predicted neighbours of this pass: all of them for water, the water ones
// for solids (the pairs pbfB uses, simkernels.js:457-458).
__global__ void XPBI_LB_PBF k_pbfA(Bufs b, int k, int flags) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  const Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  if (!pbfActive(S, k) || ((flags & kRerun) && !b.rerun[sceneIndex(b, cx)])) return;
  const float4* __restrict__ xcS = b.xc;
  const float4 pi = b.posS[i];
  const bool iWater = waterW(pi.w);
  if (!iWater) {
    // a solid only pairs with water here; candidates come from its 27 cells,
    // so with no water particle in them there is nothing to record
    const I3 cc = cellCoord(S, xyz(pi));
    bool near = false;
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
          const int x = cc.x + dx, y = cc.y + dy, z = cc.z + dz;
          if (x >= 0 && x < S.dims[0] && y >= 0 && y < S.dims[1] && z >= 0 && z < S.dims[2])
            near |= __ldg(b.cellWater + S.cellBase + cellIndex(S, x, y, z)) != 0;
        }
    if (!near) {
      b.nbrPCount[i] = 0u;
      b.pbfLam[i] = 0.f;
      b.pbfRec[i] = make_float4(0.f, 0.f, 0.f, 0.f);  // no PBF pair reads it
      return;
    }
  }
  const V3 xci = xyz(xcS[i]);
  const float s2 = S.support2;
  // the water flag is the sign bit of xc.w (the sorted pos.w)
  const uint32_t cnt =
      iWater ? recordCandidates(S, b.cellStart, xyz(pi), i, listOf(b.nbrP, i),
                                [&](uint32_t j, uint32_t& e) {  // water pairs with everything
                                  const float4 c = ldg(xcS + j);
                                  const V3 d = xci - xyz(c);
                                  e = j | (__float_as_uint(c.w) & kWaterBit);
                                  return dot(d, d) < s2;
                                })
             : recordCandidates(S, b.cellStart, xyz(pi), i, listOf(b.nbrP, i),
                                [&](uint32_t j, uint32_t& e) {  // a solid with water only
                                  const float4 c = ldg(xcS + j);
                                  const V3 d = xci - xyz(c);
                                  e = j | kWaterBit;
                                  return waterW(c.w) && dot(d, d) < s2;
                                });
  const uint32_t stored = cnt <= kNbrCap ? cnt : kNbrOverflow;
  b.nbrPCount[i] = stored;
  if (!iWater) {
    b.pbfLam[i] = 0.f;
    b.pbfRec[i] = make_float4(xci.x, xci.y, xci.z, 0.f);
    return;
  }
  const MatDev& m = cx.mats[matOfW(pi.w)];
  const float rho0 = m.density;
  const float invRho0 = __frcp_rn(rho0);
  float rho = m.mass * S.w00;
  V3 gradSum = splat(0.f);
  float grad2 = 0.f;
  auto body = [&](uint32_t, bool, const float4& c) {
    const V3 dxv = xci - xyz(c);
    const float r2 = dot(dxv, dxv);
    const float mb = cx.mats[matOfW(c.w)].mass;
    rho = rho + mb * poly6Fast(S, r2);
    const V3 g = spikyGradFast(S, dxv, r2) * (mb * invRho0);
    gradSum = gradSum + g;
    grad2 = grad2 + dot(g, g);
  };
  if (stored != kNbrOverflow) {
    forList(listOf(b.nbrP, i), stored, [&](uint32_t j) { return ldg(xcS + j); }, body);
  } else {
    forRows(S, b.cellStart, xyz(pi), [&](uint32_t beg, uint32_t end) {
#pragma unroll 1
      for (uint32_t j = beg; j < end; ++j) {
        if (j == i) continue;
        const float4 c = ldg(xcS + j);
        const V3 d = xci - xyz(c);
        if (dot(d, d) < s2) body(j, waterW(c.w), c);
      }
    });
  }
  const float C = fmaxf(rho * invRho0 - 1.f, 0.f);
  const float lam = -C / (grad2 + dot(gradSum, gradSum) + S.pbfEps);
  b.pbfLam[i] = lam;
  b.pbfRec[i] = make_float4(xci.x, xci.y, xci.z, lam);
}

struct PBData {
  float4 c;
  float lb;
};

// ---------------------------------------------------------------- pbfB
// PBF position correction with s_corr (simkernels.js:441-477) over pbfA's
// record of predicted neighbours.
__global__ void XPBI_LB_PBF k_pbfB(Bufs b, int k, const float4* velIn, float4* velOut, int flags) {
  // blocks run last to first: the pass starts where pbfA ended, on
  // slots whose data is still in L2
  const uint32_t i = (gridDim.x - 1u - blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  const Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  const float4 vi4 = velIn[i];
  if (!pbfActive(S, k) || ((flags & kRerun) && !b.rerun[sceneIndex(b, cx)])) {
    velOut[i] = vi4;
    return;
  }
  const float4* __restrict__ xcS = b.xc;
  const float* __restrict__ lam = b.pbfLam;
  const float4 pi = b.posS[i];
  const uint32_t mi = matOfW(pi.w);
  const V3 xci = xyz(xcS[i]);
  V3 dp = splat(0.f);
  const float li = lam[i];
  const bool iWater = waterW(pi.w);
  const MatDev& mWi = cx.mats[mi];
  auto gather = [&](uint32_t j) { return PBData{ldg(xcS + j), ldg(lam + j)}; };
  auto term = [&](V3 xcb, float lb, float mpd) {
    const V3 dxv = xci - xcb;
    const float r2 = dot(dxv, dxv);
    const float x = poly6Fast(S, r2) * S.invW0;
    const float x2 = x * x;
    const float sCorr = -S.sCorrK * (x2 * x2);
    dp = dp + (li + lb + sCorr) * spikyGradFast(S, dxv, r2) * mpd;
  };
  auto body = [&](uint32_t, bool jWater, const PBData& d) {
    const MatDev& mw = jWater ? cx.mats[matOfW(d.c.w)] : mWi;  // a water material
    term(xyz(d.c), d.lb, mw.massPerDensity);
  };
  const uint32_t cnt = b.nbrPCount[i];
  if (cnt != kNbrOverflow && S.waterMpd > 0.f) {
    // one water material: every pair weighs by its mass / density, and one
    // gather of pbfA's record (predicted position, multiplier) serves a pair
    const float mpd = S.waterMpd;
    forList(listOf(b.nbrP, i), cnt, [&](uint32_t j) { return ldg(b.pbfRec + j); },
            [&](uint32_t, bool, const float4& r) { term(xyz(r), r.w, mpd); });
  } else if (cnt != kNbrOverflow) {
    forList(listOf(b.nbrP, i), cnt, gather, body);
  } else {
    forRows(S, b.cellStart, xyz(pi), [&](uint32_t beg, uint32_t end) {
#pragma unroll 1
      for (uint32_t j = beg; j < end; ++j) {
        if (j == i) continue;
        const float4 c = ldg(xcS + j);
        const bool jWater = waterW(c.w);
        if (!(iWater || jWater)) continue;
        const V3 d = xci - xyz(c);
        if (dot(d, d) < S.support2) body(j, jWater, gather(j));
      }
    });
  }
  const float scale = iWater ? 1.f : 0.5f;
  V3 v = xyz(vi4) + dp * (scale / S.dt);
  // active set: a water particle's boundary, which the next solveB would
  // apply to the velocity this pass leaves (its only work on water), is
  // applied here from the same inputs, so that solveB need not visit water
  if ((flags & kInPlace) && iWater) v = applyBoundary(S, xyz(pi) + S.dt * v, v, xyz(pi), mWi.boundFriction);
  velOut[i] = make_float4(v.x, v.y, v.z, vi4.w);
  // active set: the next iteration revisits a solid this pass moved and its
  // solid neighbours, whose constraint and contact inputs it is
  if ((flags & kMarkMoved) && !iWater) {
    const V3 dvel = v - xyz(vi4);
    if (dot(dvel, dvel) > b.thr[3 * (uint32_t)(cx.scene - b.scenes) + 2]) {
      uint8_t* __restrict__ dn = b.dirty[(k + 1) & 1];
      dn[i] = 1;
      markSolidNbrs(b, cx, i, xyz(pi), dn);
    }
  }
}

// ---------------------------------------------------------------- xsph
// simkernels.js:480-507
__global__ void XPBI_LB_UPDATE k_xsph(Bufs b, const float4* __restrict__ velIn,
                                                    float4* __restrict__ velOut) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  const Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  const float4* __restrict__ posS = b.posS;
  const float4 pi = posS[i];
  const V3 xi = xyz(pi);
  const float4 vi4 = velIn[i];
  const V3 vi = xyz(vi4);
  const bool iWater = waterW(pi.w);
  V3 acc = splat(0.f);
  forNbrs(
      b, cx, i, xi, [&](uint32_t j) { return PV{ldg(posS + j), ldg(velIn + j)}; },
      [&](uint32_t, bool jWater, const PV& d) {
        if (jWater != iWater) return;
        const V3 dxv = xi - xyz(d.p);
        acc = acc + d.v.w * (xyz(d.v) - vi) * kernelWFast(S, dot(dxv, dxv));
      },
      [iWater](uint32_t e) { return ((e & kWaterBit) != 0u) == iWater; });  // same phase only
  float c = S.xsphC;
  if (iWater) c = S.xsphC * 10.f;
  const V3 v = vi + c * acc;
  velOut[i] = make_float4(v.x, v.y, v.z, vi4.w);
}

// ---------------------------------------------------------------- updateF + integrate
// Final F with return mapping (simkernels.js:510-525) fused with the CFL
// clamp and position update (simkernels.js:528-542). Outputs go to the
// "current" arrays, so neighbours still read the unclamped sorted inputs.
// The plastic update of F from the velocity gradient (simkernels.js:510-525):
// trial F, SVD, return map, the projected F. Compiled once, not inlined:
// the update kernel's sweep then keeps its registers (0.424 -> 0.401 ms per
// 4M-particle substep, the same bits).
__device__ __noinline__ M3 plasticUpdate(const SceneDev& S, const M3& gradV, const M3& F0, const MatDev& m, float st,
                                         float& stOut) {
  const M3 Ftr = mul(madd(mident(), mscale(gradV, S.dt)), F0);
  const SVD sv = svd3Fast(Ftr);
  const V3 sig = returnMap(sv.sig, m, st, S.dt, stOut);
  return diagMul(sv.U, safeSig(sig), sv.V);
}
__global__ void XPBI_LB_UPDATE k_updateF_integrate(Bufs b, const float4* __restrict__ velIn) {
  // blocks run last to first: the pass starts where xsph ended, on
  // slots whose data is still in L2
  const uint32_t i = (gridDim.x - 1u - blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  const Ctx cx = ctxOf(b, i);
  const SceneDev& S = *cx.scene;
  const float4 pi = b.posS[i];
  const uint32_t mi = matOfW(pi.w);
  const float4 vi4 = velIn[i];
  const float st = b.stateS[i];
  M3 Fn = loadM(b.FS, b.N, i);
  float stOut = st;
  if (!waterW(pi.w)) {
    const MatDev m = hardenedMat(cx.mats[mi], st);
    const M3 gradV = velocityGradient(b, cx, i, xyz(pi), xyz(vi4), velIn);
    Fn = plasticUpdate(S, gradV, Fn, m, st, stOut);
  }
  storeM(b.F, b.N, i, Fn);
  b.state[i] = stOut;
  V3 v = xyz(vi4);
  const float vl = length(v);
  if (vl > S.vmaxCFL) v = v * (S.vmaxCFL / vl);
  b.vel[i] = make_float4(v.x, v.y, v.z, vi4.w);
  V3 x = xyz(pi) + S.dt * v;
  x = v3(clampf(x.x, S.dmin[0], S.dmax[0]), clampf(x.y, S.dmin[1], S.dmax[1]), clampf(x.z, S.dmin[2], S.dmax[2]));
  b.pos[i] = make_float4(x.x, x.y, x.z, fabsf(pi.w));
}

// ---------------------------------------------------------------- device loop
// Whether any scene still iterates at iteration k: not stopped by its
// residuals and below its iteration cap (one block; every thread returns it).
__device__ __forceinline__ bool anyIterating(const Bufs& b, int k) {
  bool run = false;
  for (uint32_t s = threadIdx.x; s < b.S; s += blockDim.x)
    run |= !b.done[s] && k < b.scenes[s].iterations;
  return __syncthreads_or(run) != 0;
}
__global__ void k_loop_begin(Bufs b, int k0, cudaGraphConditionalHandle h) {
  const bool run = anyIterating(b, k0);
  if (threadIdx.x == 0) {
    *b.kIter = k0;
    cudaGraphSetConditional(h, run ? 1u : 0u);
  }
}
__global__ void k_loop_next(Bufs b, cudaGraphConditionalHandle h) {
  const int k = *reinterpret_cast<volatile const int*>(b.kIter) + 1;
  const bool run = anyIterating(b, k);  // its barrier orders every read of kIter before the write
  if (threadIdx.x == 0) {
    *b.kIter = k;
    cudaGraphSetConditional(h, run ? 1u : 0u);
  }
}

// ---------------------------------------------------------------- plain re-solve
// The judge of an early-stopped solve: a scene that did not stop within its
// iteration cap (its residuals never reached the plain solve's tolerances)
// is re-solved with the reference solve from the substep's input. Marks
// those scenes and, inside a graph, sets the condition of the node whose
// body runs the re-solve (nothing runs when every scene stopped).
__global__ void k_judge(Bufs b, cudaGraphConditionalHandle h, int setCond) {
  bool any = false;
  for (uint32_t s = threadIdx.x; s < b.S; s += blockDim.x) {
    const bool fail = b.done[s] == 0 && b.scenes[s].residTol > 0.f && b.scenes[s].plainIterations > 0;
    b.rerun[s] = fail ? 1 : 0;
    any |= fail;
  }
  any = __syncthreads_or(any) != 0;
  if (threadIdx.x == 0 && setCond) cudaGraphSetConditional(h, any ? 1u : 0u);
}
// the re-solved scenes start again from the velocities entering iteration 0
__global__ void k_restore(Bufs b, float4* __restrict__ vel) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  const uint32_t s = b.S > 1 ? (uint32_t)b.sceneOf[i] : 0u;
  if (b.rerun[s]) vel[i] = b.vel0[i];
}
// The PBF pass's predicted positions x + dt v of every slot from the
// velocities as they stand: after an active-set iteration over worklists,
// the slots it did not visit and the ones the previous PBF pass moved hold
// older ones. The expression is solveB's when it writes them, so the
// result is the one the per-slot kernels leave.
__global__ void k_predict(Bufs b, const float4* __restrict__ vel) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.N) return;
  const SceneDev& S = *ctxOf(b, i).scene;
  const float4 pi = b.posS[i];
  const V3 xc = xyz(pi) + S.dt * xyz(vel[i]);
  b.xc[i] = make_float4(xc.x, xc.y, xc.z, pi.w);
}
__global__ void k_copy_vel(uint32_t n, const float4* __restrict__ src, float4* __restrict__ dst) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i];
}

inline unsigned grid(uint32_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }
inline unsigned gridOf(uint32_t n, int block) { return (unsigned)((n + (uint32_t)block - 1) / (uint32_t)block); }

}  // namespace

void launch_computeL(const Bufs& b, bool sums, bool features, cudaStream_t st) {
  if (features)
    k_computeL_features<<<grid(b.N), kThreads, 0, st>>>(b);
  else if (sums)
    k_computeL<true><<<grid(b.N), kThreads, 0, st>>>(b);
  else
    k_computeL<false><<<grid(b.N), kThreads, 0, st>>>(b);
}
void launch_computeL_water(const Bufs& b, cudaStream_t st) { k_computeL_water<<<grid(b.N), kThreads, 0, st>>>(b); }
template <int V>
void solveAVariant(const Bufs& b, int k, const float4* velIn, int flags, cudaStream_t st) {
  if (flags & kTrackResid)
    k_solveA<true, kSolveAMinB[V], 1, kSolveABlock[V]><<<gridOf(b.N, kSolveABlock[V]), kSolveABlock[V], 0, st>>>(
        b, k, velIn, flags);
  else
    k_solveA<false, kSolveAMinB[V], 1, kSolveABlock[V]><<<gridOf(b.N, kSolveABlock[V]), kSolveABlock[V], 0, st>>>(
        b, k, velIn, flags);
}
void launch_solveA(const Bufs& b, int k, const float4* velIn, int flags, int variant, int lanes, cudaStream_t st) {
  if (flags & kStoredC) {  // iteration 0 after computeL with features (one lane per slot)
    if (flags & kTrackResid)
      k_solveA_stored<true><<<grid(b.N), kThreads, 0, st>>>(b, velIn, flags);
    else
      k_solveA_stored<false><<<grid(b.N), kThreads, 0, st>>>(b, velIn, flags);
    return;
  }
  if (lanes == 4) {  // small scenes: four lanes per slot, the allocator's register choice
    const uint32_t threads = 4u * b.N;
    if (flags & kTrackResid)
      k_solveA<true, 0, 4><<<grid(threads), kThreads, 0, st>>>(b, k, velIn, flags);
    else
      k_solveA<false, 0, 4><<<grid(threads), kThreads, 0, st>>>(b, k, velIn, flags);
    return;
  }
  if (lanes == 2) {
    const uint32_t threads = 2u * b.N;
    if (flags & kTrackResid)
      k_solveA<true, 0, 2><<<grid(threads), kThreads, 0, st>>>(b, k, velIn, flags);
    else
      k_solveA<false, 0, 2><<<grid(threads), kThreads, 0, st>>>(b, k, velIn, flags);
    return;
  }
  switch (variant) {
    case 1: solveAVariant<1>(b, k, velIn, flags, st); break;
    case 2: solveAVariant<2>(b, k, velIn, flags, st); break;
    case 3: solveAVariant<3>(b, k, velIn, flags, st); break;
    case 4: solveAVariant<4>(b, k, velIn, flags, st); break;
    case 5: solveAVariant<5>(b, k, velIn, flags, st); break;
    default: solveAVariant<0>(b, k, velIn, flags, st); break;
  }
}
void launch_warm_from_net(const Bufs& b, cudaStream_t st) { k_warm_from_net<<<grid(b.N), kThreads, 0, st>>>(b); }
void launch_warm_from_prev(const Bufs& b, cudaStream_t st) { k_warm_from_prev<<<grid(b.N), kThreads, 0, st>>>(b); }
void launch_resid_reduce(const Bufs& b, int k, bool warm, cudaStream_t st) {
  k_resid<<<dim3(residBlocks(b.maxSceneN), b.S), kResidThreads, 0, st>>>(b, k, warm ? 1 : 0);
}
void launch_keep_lambda(const Bufs& b, cudaStream_t st) { k_keep_lambda<<<grid(b.N), kThreads, 0, st>>>(b); }
template <int V>
void solveBVariant(const Bufs& b, int k, const float4* velIn, float4* velOut, int wx, int flags, cudaStream_t st) {
  k_solveB<kSolveBMinB[V], 1, kSolveBBlock[V]><<<gridOf(b.N, kSolveBBlock[V]), kSolveBBlock[V], 0, st>>>(
      b, k, velIn, velOut, wx, flags);
}
// A grid that fills the GPU once with this kernel's resident blocks (the
// list launches loop over their lists).
inline unsigned fillGrid(const void* fn, int block) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, 0);
  return (unsigned)(std::max(1, sms) * std::max(1, per));
}
template <int V>
void solveBActiveVariant(const Bufs& b, int k, float4* vel, int wx, int flags, bool list, cudaStream_t st) {
  auto fn = k_solveB_active<kSolveBMinB[V], kSolveBBlock[V]>;
  const unsigned g = list ? fillGrid((const void*)fn, kSolveBBlock[V]) : gridOf(b.N, kSolveBBlock[V]);
  fn<<<g, kSolveBBlock[V], 0, st>>>(b, k, vel, wx, flags, list ? 1 : 0);
}
template <int V>
void solveAListVariant(const Bufs& b, int k, const float4* velIn, int flags, cudaStream_t st) {
  constexpr int minB = kSolveAMinB[V];
  auto fn = k_solveA_list<minB, kSolveABlock[V]>;
  fn<<<fillGrid((const void*)fn, kSolveABlock[V]), kSolveABlock[V], 0, st>>>(b, k, velIn, flags);
}
void launch_solveB(const Bufs& b, int k, const float4* velIn, float4* velOut, bool writeXc, int flags, int variant,
                   int lanes, cudaStream_t st) {
  const int wx = writeXc ? 1 : 0;
  if (flags & (kInPlace | kActive | kMarkMoved)) {  // the active set: in place, one lane per slot
    float4* vel = velOut;
    switch (variant) {
      case 1: solveBActiveVariant<1>(b, k, vel, wx, flags, false, st); break;
      case 2: solveBActiveVariant<2>(b, k, vel, wx, flags, false, st); break;
      case 3: solveBActiveVariant<3>(b, k, vel, wx, flags, false, st); break;
      case 4: solveBActiveVariant<4>(b, k, vel, wx, flags, false, st); break;
      default: solveBActiveVariant<0>(b, k, vel, wx, flags, false, st); break;
    }
    return;
  }
  if (lanes == 4) {
    k_solveB<0, 4><<<grid(4u * b.N), kThreads, 0, st>>>(b, k, velIn, velOut, wx, flags);
    return;
  }
  if (lanes == 2) {
    k_solveB<0, 2><<<grid(2u * b.N), kThreads, 0, st>>>(b, k, velIn, velOut, wx, flags);
    return;
  }
  switch (variant) {
    case 1: solveBVariant<1>(b, k, velIn, velOut, wx, flags, st); break;
    case 2: solveBVariant<2>(b, k, velIn, velOut, wx, flags, st); break;
    case 3: solveBVariant<3>(b, k, velIn, velOut, wx, flags, st); break;
    case 4: solveBVariant<4>(b, k, velIn, velOut, wx, flags, st); break;
    default: solveBVariant<0>(b, k, velIn, velOut, wx, flags, st); break;
  }
}
void launch_loop_begin(const Bufs& b, int k0, cudaGraphConditionalHandle h, cudaStream_t st) {
  k_loop_begin<<<1, 256, 0, st>>>(b, k0, h);
}
void launch_loop_next(const Bufs& b, cudaGraphConditionalHandle h, cudaStream_t st) {
  k_loop_next<<<1, 256, 0, st>>>(b, h);
}
void launch_compact(const Bufs& b, int k, int which, cudaStream_t st) {
  k_compact<<<gridOf((b.N + kCompactSlots - 1) / kCompactSlots, kCompactThreads), kCompactThreads, 0, st>>>(b, k,
                                                                                                       which);
}
void launch_solveA_list(const Bufs& b, int k, const float4* velIn, int flags, int variant, cudaStream_t st) {
  switch (variant) {
    case 1: solveAListVariant<1>(b, k, velIn, flags, st); break;
    case 2: solveAListVariant<2>(b, k, velIn, flags, st); break;
    case 3: solveAListVariant<3>(b, k, velIn, flags, st); break;
    case 4: solveAListVariant<4>(b, k, velIn, flags, st); break;
    case 5: solveAListVariant<5>(b, k, velIn, flags, st); break;
    default: solveAListVariant<0>(b, k, velIn, flags, st); break;
  }
}
void launch_solveB_list(const Bufs& b, int k, float4* vel, int flags, int variant, cudaStream_t st) {
  switch (variant) {
    case 1: solveBActiveVariant<1>(b, k, vel, 0, flags, true, st); break;
    case 2: solveBActiveVariant<2>(b, k, vel, 0, flags, true, st); break;
    case 3: solveBActiveVariant<3>(b, k, vel, 0, flags, true, st); break;
    case 4: solveBActiveVariant<4>(b, k, vel, 0, flags, true, st); break;
    default: solveBActiveVariant<0>(b, k, vel, 0, flags, true, st); break;
  }
}
void launch_pbfA(const Bufs& b, int k, const float4* velIn, int flags, cudaStream_t st) {
  (void)velIn;  // predicted positions were stored by the preceding solveB
  k_pbfA<<<grid(b.N), kThreads, 0, st>>>(b, k, flags);
}
void launch_judge(const Bufs& b, cudaGraphConditionalHandle h, bool setCond, cudaStream_t st) {
  k_judge<<<1, 256, 0, st>>>(b, h, setCond ? 1 : 0);
}
void launch_restore(const Bufs& b, float4* vel, cudaStream_t st) { k_restore<<<grid(b.N), kThreads, 0, st>>>(b, vel); }
void launch_predict(const Bufs& b, const float4* vel, cudaStream_t st) { k_predict<<<grid(b.N), kThreads, 0, st>>>(b, vel); }
void launch_copy_vel(const Bufs& b, const float4* src, float4* dst, cudaStream_t st) {
  k_copy_vel<<<grid(b.N), kThreads, 0, st>>>(b.N, src, dst);
}
void launch_pbfB(const Bufs& b, int k, const float4* velIn, float4* velOut, int flags, cudaStream_t st) {
  k_pbfB<<<grid(b.N), kThreads, 0, st>>>(b, k, velIn, velOut, flags);
}
void launch_xsph(const Bufs& b, const float4* velIn, float4* velOut, cudaStream_t st) {
  k_xsph<<<grid(b.N), kThreads, 0, st>>>(b, velIn, velOut);
}
void launch_updateF_integrate(const Bufs& b, const float4* velIn, cudaStream_t st) {
  k_updateF_integrate<<<grid(b.N), kThreads, 0, st>>>(b, velIn);
}

}  // namespace xpbi
