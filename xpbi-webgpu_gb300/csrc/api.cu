// C ABI of libxpbi (declared in include/xpbi.h): the GB300 counterpart of the
// reference's `Simulation` class (web/js/sim.js:9-273) and of the frame
// loop's substep loop (web/js/main.js:385-415).
//
// Host packing here follows sim.js exactly where it feeds the kernels: grid
// sizing in f64 (sim.js:20-26), material derivation mu/lambda/mass in f64
// (sim.js:84-99), Params words (sim.js:159-186). Constants that the WGSL
// re-derives per call (kernel normalisations, alpha-tilde, caps) are formed
// once per writeParams in f32 with the same operation order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "render.h"
#include "xpbi.h"
#include "xpbi_internal.h"

using namespace xpbi;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define XPBI_CK(call)                                                                      \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      return fail(e_ == cudaErrorMemoryAllocation ? XPBI_ERR_OOM : XPBI_ERR_CUDA,          \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                     \
    }                                                                                      \
  } while (0)

struct SceneHost {
  uint32_t n = 0, pBase = 0, cellBase = 0, numCells = 0;
  double h = 0, support = 0, V0 = 0;
  double dmin[3] = {0, 0, 0}, dmax[3] = {0, 0, 0};
  double origin[3] = {0, 0, 0};
  int dims[3] = {0, 0, 0};
  xpbi_material mats[kMaxMats];
  uint32_t nMats = 0;
  uint32_t matCount[kMaxMats] = {0};  // particles per material at creation
  xpbi_params params;
  int iterations = 0, hasWater = 0;
};

float f32(double x) { return (float)x; }
uint32_t bits(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
}

// sim.js:20-26
int sizeGrid(const xpbi_scene_desc& d, SceneHost& s) {
  if (!(d.h > 0) || !std::isfinite(d.h)) return fail(XPBI_ERR_INVALID, "scene h must be positive and finite");
  s.h = d.h;
  s.support = 2 * d.h;
  s.V0 = std::pow(d.h, 3.0);
  const double cs = s.support;
  const int pad = 2;
  double cells = 1;
  for (int k = 0; k < 3; ++k) {
    if (!(d.domain_max[k] > d.domain_min[k])) return fail(XPBI_ERR_INVALID, "scene domain_max must exceed domain_min");
    s.dmin[k] = d.domain_min[k];
    s.dmax[k] = d.domain_max[k];
    s.origin[k] = d.domain_min[k] - pad * cs;
    double dim = std::ceil((d.domain_max[k] - d.domain_min[k]) / cs) + 2 * pad;
    if (!(dim >= 1) || dim > 1e6) return fail(XPBI_ERR_INVALID, "scene grid dimension out of range");
    s.dims[k] = (int)dim;
    cells *= dim;
  }
  if (cells > 2147483647.0) return fail(XPBI_ERR_INVALID, "scene grid has too many cells");
  s.numCells = (uint32_t)cells;
  return XPBI_OK;
}

void defaultParams(const SceneHost& s, xpbi_params& p) {
  std::memset(&p, 0, sizeof(p));
  p.dt = 0;
  for (int k = 0; k < 3; ++k) {
    p.domain_min[k] = (float)s.dmin[k];
    p.domain_max[k] = (float)s.dmax[k];
  }
  p.gravity[1] = -9.8f;  // scenes.js:86
  p.xsph_c = 0.01f;
  p.omega = 0.5f;
  p.contact_omega = 0.4f;
  p.pbf_eps = 100.f;
  p.s_corr_k = 1e-4f;
  p.k_damp = 0.4f;
  p.pbf_iterations = -1;
}

// sim.js:84-99 (one material into 16 words)
void packMaterial(const xpbi_material& m, double V0, uint32_t* o) {
  const double E = m.E, nu = m.nu;
  const double mu = E / (2 * (1 + nu));
  const double lam = E * nu / ((1 + nu) * (1 - 2 * nu));
  o[0] = bits(f32(mu));
  o[1] = bits(f32(lam));
  o[2] = bits(f32(m.density));
  o[3] = m.kind;
  o[4] = bits(f32(m.p0));
  o[5] = bits(f32(m.p1));
  o[6] = bits(f32(m.p2));
  o[7] = bits(f32(m.p3));
  o[8] = bits(m.color[0]);
  o[9] = bits(m.color[1]);
  o[10] = bits(m.color[2]);
  o[11] = bits(1.f);
  o[12] = bits(f32(m.bound_friction));
  o[13] = bits(f32(m.density * V0));
  o[14] = 0;
  o[15] = 0;
}

// sim.js:159-186
void packParams(const SceneHost& s, const xpbi_params& p, uint32_t* w) {
  std::memset(w, 0, 4 * XPBI_PARAMS_WORDS);
  for (int k = 0; k < 3; ++k) {
    w[k] = bits(f32(s.origin[k]));
    w[4 + k] = (uint32_t)s.dims[k];
    w[8 + k] = bits(p.domain_min[k]);
    w[12 + k] = bits(p.domain_max[k]);
    w[16 + k] = bits(p.gravity[k]);
    w[20 + k] = bits(p.collider_pos[k]);
    w[24 + k] = bits(p.collider_vel[k]);
  }
  w[3] = bits(f32(s.support));
  w[7] = s.numCells;
  w[11] = bits(p.dt);
  w[15] = bits(f32(s.h));
  w[19] = bits(f32(s.support));
  w[23] = bits(p.collider_r);
  w[27] = bits(p.collider_active ? 1.f : 0.f);
  w[28] = s.n;
  w[29] = bits(f32(s.V0));
  w[30] = bits(p.xsph_c);
  w[31] = bits(p.omega);
  w[32] = bits(p.pbf_eps);
  w[33] = bits(p.s_corr_k);
  w[34] = bits(p.time);
  w[35] = bits(p.contact_omega);
  w[36] = bits(p.k_damp);
}

float wf(const uint32_t* w, int k) {
  float x;
  std::memcpy(&x, &w[k], 4);
  return x;
}

// Device uniforms from the packed words. Every float here is read back from
// the packed words, so kernels see exactly the f32 values the WGSL would.
void buildSceneDev(const SceneHost& s, uint32_t sceneIdx, SceneDev& d, MatDev* md) {
  uint32_t w[XPBI_PARAMS_WORDS], m[kMaxMats * XPBI_MATERIAL_WORDS];
  packParams(s, s.params, w);
  std::memset(m, 0, sizeof(m));
  for (uint32_t i = 0; i < s.nMats; ++i) packMaterial(s.mats[i], s.V0, m + 16 * i);
  std::memset(&d, 0, sizeof(d));
  for (int k = 0; k < 3; ++k) {
    d.origin[k] = wf(w, k);
    d.dims[k] = (int)w[4 + k];
    d.dmin[k] = wf(w, 8 + k);
    d.dmax[k] = wf(w, 12 + k);
    d.grav[k] = wf(w, 16 + k);
    d.colPos[k] = wf(w, 20 + k);
    d.colVel[k] = wf(w, 24 + k);
  }
  d.cs = wf(w, 3);
  d.numCells = w[7];
  d.cellBase = s.cellBase;
  d.pBase = s.pBase;
  d.n = s.n;
  d.matBase = sceneIdx * kMaxMats;
  d.dt = wf(w, 11);
  d.h = wf(w, 15);
  d.support = wf(w, 19);
  d.colR = wf(w, 23);
  d.colActive = wf(w, 27);
  d.V0 = wf(w, 29);
  d.xsphC = wf(w, 30);
  d.omega = wf(w, 31);
  d.pbfEps = wf(w, 32);
  d.sCorrK = wf(w, 33);
  d.contactOmega = wf(w, 35);
  d.kDamp = wf(w, 36);
  const float h = d.h, H = d.support, dt = d.dt;
  d.support2 = H * H;
  d.sigW = 21.f / ((float)(16.0 * 3.14159265) * h * h * h);
  d.poly6C = 315.f / ((float)(64.0 * 3.14159265) * powf(H, 9.f));
  d.spikyC = -45.f / ((float)3.14159265 * powf(H, 6.f));
  {
    const float x = H * H - 0.f * 0.f;
    d.w00 = d.poly6C * x * x * x;
  }
  {
    const float r = 0.2f * H;
    if (r >= H) d.w0 = 0.f;
    else {
      const float x = H * H - r * r;
      d.w0 = d.poly6C * x * x * x;
    }
  }
  d.invH = 1.f / h;
  d.invW0 = 1.f / fmaxf(d.w0, 1e-12f);
  d.alphaT = (1.f / d.V0) / (dt * dt);
  d.minD = 0.75f * h;
  d.vmaxCFL = 0.45f * H / dt;
  d.dvCap = 0.2f * H / dt;
  d.iterations = s.iterations;
  d.pbfIterations = s.params.pbf_iterations;
  d.pbfUntil = s.params.pbf_iterations < 0 ? s.iterations : std::min(s.iterations, s.params.pbf_iterations);
  d.plainIterations = s.iterations;
  d.hasWater = s.hasWater;
  for (int i = 0; i < kMaxMats; ++i) {
    const uint32_t* q = m + 16 * i;
    MatDev& M = md[i];
    std::memset(&M, 0, sizeof(M));
    M.mu = wf(q, 0);
    M.lam = wf(q, 1);
    M.density = wf(q, 2);
    M.kind = q[3];
    M.p0 = wf(q, 4);
    M.p1 = wf(q, 5);
    M.p2 = wf(q, 6);
    M.p3 = wf(q, 7);
    M.boundFriction = wf(q, 12);
    M.mass = wf(q, 13);
    M.massPerDensity = M.density != 0.f ? M.mass / M.density : 0.f;
  }
  // PBF pairs weight by the water particle's mass / density; with one water
  // material it is a scene constant
  d.waterMpd = 0.f;
  int nWater = 0;
  for (uint32_t i = 0; i < s.nMats && i < (uint32_t)kMaxMats; ++i)
    if (md[i].kind == kKindWater) {
      ++nWater;
      d.waterMpd = md[i].massPerDensity;
    }
  if (nWater != 1) d.waterMpd = 0.f;
}

int validateScene(const xpbi_scene_desc* d) {
  if (!d) return fail(XPBI_ERR_INVALID, "scene descriptor is NULL");
  if (d->n > 0 && (!d->positions || !d->mat_ids)) return fail(XPBI_ERR_INVALID, "positions and mat_ids are required");
  if (d->n_materials < 1 || d->n_materials > (uint32_t)kMaxMats || !d->materials)
    return fail(XPBI_ERR_INVALID, "n_materials must be 1..8 with a materials array");
  for (uint32_t i = 0; i < d->n_materials; ++i)
    if (d->materials[i].kind > XPBI_WATER) return fail(XPBI_ERR_INVALID, "material kind out of range");
  for (uint32_t i = 0; i < d->n; ++i)
    if (d->mat_ids[i] >= d->n_materials) return fail(XPBI_ERR_INVALID, "mat_ids entry >= n_materials");
  return XPBI_OK;
}

}  // namespace

namespace xpbi {
int setError(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace xpbi

struct xpbi_sim {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t capture = nullptr;
  Bufs b{};
  std::vector<SceneHost> sc;
  std::vector<SceneDev> sdev;
  std::vector<MatDev> mdev;
  std::vector<uint32_t> matWordsHost;
  // page-locked staging of the uniforms, a ring of kUploadRing slots each
  // reused once its copy completed: a copy from pageable memory would first
  // wait for the stream's earlier work, so a frame's writeParams + step
  // could not be queued while the previous substep runs
  static constexpr int kUploadRing = 3;
  uint8_t* upHost[kUploadRing] = {};
  cudaEvent_t upDone[kUploadRing] = {};
  size_t upCap = 0;
  int upNext = 0;
  uint32_t* matWords = nullptr;  // packed reference material table [S*128] (renderer binding)
  bool dirty = true;
  bool fresh = true;
  bool waterLPending = false;  // a substep ran since the water particles' L was last formed
  // asynchronous position read-back (xpbi_read_positions_async): a copy
  // stream that waits for the work enqueued so far; a substep's position
  // update waits for the copies (an external event wait, also in graphs)
  cudaStream_t copy = nullptr;
  cudaStream_t loop = nullptr;  // captures the body of the device loop (early-stopped solves in a graph)
  cudaEvent_t evWork = nullptr, evCopy = nullptr;
  bool copyPending = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  std::string gkey;
  std::vector<void*> allocs;
  // solver mode: 0 plain (reference), 1 network warm start, 2 previous-multiplier warm start
  int mode = 0;
  float residTol = 0.f;     // early stop tolerance relative to |C(v_pred)|; <= 0 off
  float residTolC = 0.f;    // the contact residual's tolerance
  bool track = false;       // residual history per iteration
  float activeShare = 0.f;  // active set: share of the residual budget settled slots may hold (0: off)
  int maxIters = 0;         // an early-stopped solve may iterate up to this many times (0: the scene's count)
  bool features = false;    // compute network features every substep (training logs)
  bool netLoaded = false;
  float* netParams = nullptr;
  int* netErr = nullptr;
  // register-allocation variants of solveA / solveB (xpbi_autotune)
  int tuneA = 0, tuneB = 0;
  int lanesMode = 0;  // lanes per slot in solveA / solveB: 0 by size, 1 or 4
  // headless renderer targets (xpbi_render), sized on demand
  unsigned long long* renderImg = nullptr;
  uint32_t* renderRgba = nullptr;
  size_t renderPixels = 0;
};

namespace {

template <class T>
int alloc(xpbi_sim* s, T** p, size_t count) {
  void* q = nullptr;
  size_t bytes = std::max<size_t>(count * sizeof(T), 256);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) return fail(XPBI_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  s->allocs.push_back(q);
  *p = (T*)q;
  return XPBI_OK;
}

#define XPBI_TRY(x)               \
  do {                            \
    int r_ = (x);                 \
    if (r_ != XPBI_OK) return r_; \
  } while (0)

void destroyAll(xpbi_sim* s) {
  for (int j = 0; j < xpbi_sim::kUploadRing; ++j) {  // no copy may still read a staging slot
    if (s->upDone[j]) cudaEventSynchronize(s->upDone[j]);
    if (s->upHost[j]) cudaFreeHost(s->upHost[j]);
    if (s->upDone[j]) cudaEventDestroy(s->upDone[j]);
  }
  if (s->gexec) cudaGraphExecDestroy(s->gexec);
  if (s->graph) cudaGraphDestroy(s->graph);
  for (void* p : s->allocs) cudaFree(p);
  if (s->renderImg) cudaFree(s->renderImg);
  if (s->renderRgba) cudaFree(s->renderRgba);
  if (s->own) cudaStreamDestroy(s->own);
  if (s->capture) cudaStreamDestroy(s->capture);
  if (s->copy) cudaStreamDestroy(s->copy);
  if (s->loop) cudaStreamDestroy(s->loop);
  if (s->evWork) cudaEventDestroy(s->evWork);
  if (s->evCopy) cudaEventDestroy(s->evCopy);
}

// Work outside the substep that rewrites the positions waits for the
// asynchronous read-backs enqueued before it.
void drainCopies(xpbi_sim* s) {
  if (!s->copyPending) return;
  cudaStreamWaitEvent(s->stream, s->evCopy, 0);
  s->copyPending = false;
}

int upload(xpbi_sim* s) {
  if (!s->dirty) return XPBI_OK;
  const uint32_t S = (uint32_t)s->sc.size();
  s->sdev.resize(S);
  s->mdev.resize((size_t)S * kMaxMats);
  s->matWordsHost.assign((size_t)S * kMaxMats * XPBI_MATERIAL_WORDS, 0u);
  for (uint32_t i = 0; i < S; ++i) {
    buildSceneDev(s->sc[i], i, s->sdev[i], &s->mdev[(size_t)i * kMaxMats]);
    s->sdev[i].residTol = s->residTol;
    s->sdev[i].residTolC = s->residTolC;
    s->sdev[i].asShare = s->activeShare;
    if (s->residTol > 0.f && s->maxIters > s->sc[i].iterations) s->sdev[i].iterations = s->maxIters;
    uint32_t solids = 0;
    for (uint32_t m = 0; m < s->sc[i].nMats; ++m)
      if (s->sc[i].mats[m].kind != XPBI_WATER) solids += s->sc[i].matCount[m];
    s->sdev[i].nSolid = solids;
    for (uint32_t m = 0; m < s->sc[i].nMats; ++m)
      packMaterial(s->sc[i].mats[m], s->sc[i].V0, &s->matWordsHost[((size_t)i * kMaxMats + m) * XPBI_MATERIAL_WORDS]);
  }
  const size_t bS = sizeof(SceneDev) * S, bM = sizeof(MatDev) * s->mdev.size(), bW = 4 * s->matWordsHost.size();
  const size_t oM = (bS + 255) & ~size_t(255), oW = (oM + bM + 255) & ~size_t(255), need = oW + bW;
  if (need > s->upCap) {  // (re)allocate the ring: wait for the copies that read the old one
    for (int j = 0; j < xpbi_sim::kUploadRing; ++j) {
      if (s->upDone[j]) XPBI_CK(cudaEventSynchronize(s->upDone[j]));
      if (s->upHost[j]) cudaFreeHost(s->upHost[j]);
      s->upHost[j] = nullptr;
    }
    s->upCap = 0;
    for (int j = 0; j < xpbi_sim::kUploadRing; ++j) {
      if (cudaMallocHost(reinterpret_cast<void**>(&s->upHost[j]), need) != cudaSuccess)
        return fail(XPBI_ERR_OOM, "page-locked staging of the uniforms");
      if (!s->upDone[j]) XPBI_CK(cudaEventCreateWithFlags(&s->upDone[j], cudaEventDisableTiming));
    }
    s->upCap = need;
  }
  const int j = s->upNext;
  s->upNext = (j + 1) % xpbi_sim::kUploadRing;
  XPBI_CK(cudaEventSynchronize(s->upDone[j]));  // this slot's last copy, kUploadRing uploads ago
  uint8_t* h = s->upHost[j];
  std::memcpy(h, s->sdev.data(), bS);
  std::memcpy(h + oM, s->mdev.data(), bM);
  std::memcpy(h + oW, s->matWordsHost.data(), bW);
  XPBI_CK(cudaMemcpyAsync(s->b.scenes, h, bS, cudaMemcpyHostToDevice, s->stream));
  XPBI_CK(cudaMemcpyAsync(s->b.mats, h + oM, bM, cudaMemcpyHostToDevice, s->stream));
  XPBI_CK(cudaMemcpyAsync(s->matWords, h + oW, bW, cudaMemcpyHostToDevice, s->stream));
  XPBI_CK(cudaEventRecord(s->upDone[j], s->stream));
  s->dirty = false;
  return XPBI_OK;
}

// Iterations a scene may run this substep: its own count, or for an
// early-stopped solve the larger cap of xpbi_set_max_iterations.
int effIterations(const xpbi_sim* s, const SceneHost& h) {
  return s->residTol > 0.f && s->maxIters > h.iterations ? s->maxIters : h.iterations;
}

// The substep's launch schedule: max iterations and which iterations run PBF.
struct Schedule {
  int K = 0;
  std::vector<char> pbf;
  int mode = 0;          // 0 plain, 1 network warm start, 2 previous-multiplier warm start
  bool track = false;    // residual history (includes the pass after the last iteration)
  bool reduce = false;   // per-iteration residual reductions (history or early stop)
  bool features = false; // network features at iteration 0
  bool keepLam = false;  // carry the final multipliers into the next substep
  int varA = 0, varB = 0; // solveA / solveB variants
  int lanes = 1;          // lanes per slot in solveA / solveB
  bool active = false;    // active set (work skipping) in the iterations
  bool fallback = false;  // scenes an early-stopped solve fails are re-solved plainly
  std::string key() const {
    std::string k = std::to_string(K) + ":";
    for (char c : pbf) k += c ? '1' : '0';
    k += ":" + std::to_string(mode) + (track ? "t" : "") + (reduce ? "r" : "") + (features ? "f" : "") +
         (keepLam ? "l" : "") + (active ? "a" : "") + (fallback ? "j" : "") + ":v" + std::to_string(varA) + std::to_string(varB) + ":g" +
         std::to_string(lanes);
    return k;
  }
};

Schedule schedule(const xpbi_sim* s) {
  Schedule sch;
  sch.mode = s->mode;
  sch.track = s->track;
  sch.reduce = s->track || s->residTol > 0.f;
  sch.features = s->features || s->mode == 1;
  sch.keepLam = s->mode != 0 || sch.features;
  sch.varA = s->tuneA;
  sch.varB = s->tuneB;
  if (s->lanesMode) {
    sch.lanes = s->lanesMode;
  } else {
    // the constraint kernels' work is the solid particles (water threads
    // leave at once): few of them leave the GPU idle with one lane each
    uint64_t solids = 0;
    for (const SceneHost& h : s->sc)
      for (uint32_t m = 0; m < h.nMats; ++m)
        if (h.mats[m].kind != XPBI_WATER) solids += h.matCount[m];
    sch.lanes = solids <= kFourLaneSolids ? 4 : (solids <= kTwoLaneSolids ? 2 : 1);
  }
  // the active set needs the early stop's residual sums and one lane per slot
  sch.active = s->activeShare > 0.f && s->residTol > 0.f && sch.lanes == 1;
  // an early-stopped solve that differs from the reference (a warm start or
  // the active set) is judged against the plain tolerances it was given
  sch.fallback = s->residTol > 0.f && (s->mode != 0 || sch.active);
  for (const SceneHost& h : s->sc) sch.K = std::max(sch.K, effIterations(s, h));
  sch.pbf.assign(sch.K, 0);
  for (const SceneHost& h : s->sc) {
    if (!h.hasWater) continue;
    for (int k = 0; k < h.iterations; ++k)
      if (h.params.pbf_iterations < 0 || k < h.params.pbf_iterations) sch.pbf[k] = 1;
  }
  return sch;
}

struct Recorder {
  // optional per-launch event timing (profileSubstep)
  std::vector<cudaEvent_t>* ev = nullptr;
  std::vector<std::string>* labels = nullptr;
  void mark(cudaStream_t st, const char* label) {
    if (!ev) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, st);
    ev->push_back(e);
    if (label) labels->push_back(label);
  }
};

// One active-set iteration's solve (k may be kIterDevice): the changed
// solids and the slots solveB updates compacted into lists, solveA and
// solveB over them, the residual reduction.
void enqueueListIteration(const Bufs& b, const Schedule& sch, int k, int aflags, cudaStream_t st, Recorder& R) {
  const int act = kInPlace | kMarkMoved | kActive;
  launch_compact(b, k, 0, st);
  R.mark(st, "compact");
  launch_solveA_list(b, k, b.velS[0], aflags | act, sch.varA, st);
  R.mark(st, "solveA");
  launch_compact(b, k, 1, st);
  R.mark(st, "compact");
  launch_solveB_list(b, k, b.velS[0], (sch.reduce ? kTrackResid : 0) | act, sch.varB, st);
  R.mark(st, "solveB");
  launch_resid_reduce(b, k, (aflags & kWarm) != 0, st);
  R.mark(st, "residual");
}

// Inside a stream capture: the iterations k0..K-1 of an early-stopped
// solve as a while node of the graph, whose body (one list iteration on the
// device's iteration counter) repeats until every scene stopped or reached
// its cap; no launch is spent on iterations nothing needs.
cudaError_t captureDeviceLoop(xpbi_sim* s, const Schedule& sch, int k0, int aflags, cudaStream_t st) {
  const Bufs& b = s->b;
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd);
  if (e != cudaSuccess) return e;
  cudaGraphConditionalHandle h;
  if ((e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault)) != cudaSuccess) return e;
  launch_loop_begin(b, k0, h, st);
  if ((e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd)) != cudaSuccess) return e;
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  if ((e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &p)) != cudaSuccess) return e;
  cudaGraph_t body = p.conditional.phGraph_out[0];
  if ((e = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies)) !=
      cudaSuccess)
    return e;
  if ((e = cudaStreamBeginCaptureToGraph(s->loop, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed)) !=
      cudaSuccess)
    return e;
  Recorder none;
  enqueueListIteration(b, sch, kIterDevice, aflags, s->loop, none);
  launch_loop_next(b, h, s->loop);
  cudaGraph_t out = nullptr;
  return cudaStreamEndCapture(s->loop, &out);
}

// The plain re-solve of the scenes the judge marked: their velocities back
// to vel0, then the reference schedule (lambda from 0, every slot of those
// scenes, the scenes' own iteration counts and PBF passes) with the other
// scenes' velocities copied through the ping-pong; the result ends in
// velS[in] like the solve it replaces.
void enqueuePlainResolve(xpbi_sim* s, const Schedule& sch, int in, cudaStream_t st, Recorder& R) {
  const Bufs& b = s->b;
  launch_restore(b, b.velS[in], st);
  R.mark(st, "restore");
  int cur = in;
  int K = 0;
  for (const SceneHost& h : s->sc) K = std::max(K, h.iterations);
  for (int k = 0; k < K; ++k) {
    const bool pbf = k < (int)sch.pbf.size() && sch.pbf[k];
    launch_solveA(b, k, b.velS[cur], kRerun, sch.varA, sch.lanes, st);
    R.mark(st, "solveA");
    launch_solveB(b, k, b.velS[cur], b.velS[cur ^ 1], pbf, kRerun, sch.varB, sch.lanes, st);
    R.mark(st, "solveB");
    cur ^= 1;
    if (pbf) {
      launch_pbfA(b, k, b.velS[cur], kRerun, st);
      R.mark(st, "pbfA");
      launch_pbfB(b, k, b.velS[cur], b.velS[cur ^ 1], kRerun, st);
      R.mark(st, "pbfB");
      cur ^= 1;
    }
  }
  if (cur != in) {
    launch_copy_vel(b, b.velS[cur], b.velS[in], st);
    R.mark(st, "copy");
  }
}

// Inside a stream capture: the judge, then the plain re-solve as the body
// of a conditional node the judge's kernel switches on only when a scene
// failed.
cudaError_t captureFallback(xpbi_sim* s, const Schedule& sch, int in, cudaStream_t st) {
  const Bufs& b = s->b;
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd);
  if (e != cudaSuccess) return e;
  cudaGraphConditionalHandle h;
  if ((e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault)) != cudaSuccess) return e;
  launch_judge(b, h, true, st);
  if ((e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd)) != cudaSuccess) return e;
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeIf;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  if ((e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &p)) != cudaSuccess) return e;
  cudaGraph_t body = p.conditional.phGraph_out[0];
  if ((e = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies)) !=
      cudaSuccess)
    return e;
  if ((e = cudaStreamBeginCaptureToGraph(s->loop, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed)) !=
      cudaSuccess)
    return e;
  Recorder none;
  enqueuePlainResolve(s, sch, in, s->loop, none);
  cudaGraph_t out = nullptr;
  return cudaStreamEndCapture(s->loop, &out);
}

// encodeSubstep (sim.js:220-272). Ping-pong parity is resolved on the host:
// the last writer's buffer is passed to updateF+integrate directly, so no
// copy-back is needed (the reference copies velB -> velA when odd).
cudaError_t enqueueSubstep(xpbi_sim* s, const Schedule& sch, cudaStream_t st, Recorder* rec) {
  const Bufs& b = s->b;
  Recorder none;
  Recorder& R = rec ? *rec : none;
  R.mark(st, nullptr);
  launch_count(b, st);
  R.mark(st, "count");
  launch_scan(b, st);
  R.mark(st, "scan");
  launch_scatter(b, st);
  R.mark(st, "fill");
  launch_reorder(b, sch.keepLam, st);
  R.mark(st, "reorder");
  // the velocity-free sums are read by the one-lane constraint sweeps; with
  // features (the learned solve, or features logged) the same pass also
  // stores iteration 0's constraint and the network's features
  launch_computeL(b, sch.lanes == 1 || sch.features, sch.features, st);
  R.mark(st, "computeL");
  if (sch.mode == 1) {
    mlp_forward(b.feat, b.N, b.netBlob, b.netOut, nullptr, s->netErr, st, true);
    R.mark(st, "network");
    launch_warm_from_net(b, st);
    R.mark(st, "warmstart");
  } else if (sch.mode == 2) {
    launch_warm_from_prev(b, st);
    R.mark(st, "warmstart");
  }
  if (sch.reduce) {
    cudaMemsetAsync(b.done, 0, sizeof(int) * b.S, st);
    cudaMemsetAsync(b.itersUsed, 0, sizeof(int) * b.S, st);
  }
  if (sch.active) {  // nothing is marked before iteration 0, which visits every slot
    const size_t padded = ((size_t)b.N + 15) & ~size_t(15);
    cudaMemsetAsync(b.dirty[0], 0, padded, st);
    cudaMemsetAsync(b.dirty[1], 0, padded, st);
    cudaMemsetAsync(b.bmark, 0, padded, st);
    cudaMemsetAsync(b.imp, 0, b.N, st);
    cudaMemsetAsync(b.actA, 0, sizeof(uint32_t) * kMaxResid, st);
    cudaMemsetAsync(b.actB, 0, sizeof(uint32_t) * kMaxResid, st);
  }
  const int aflags = (sch.reduce ? kTrackResid : 0) | (sch.mode != 0 ? kWarm : 0);
  if (sch.fallback)  // the plain re-solve starts from these velocities
    cudaMemcpyAsync(b.vel0, b.velS[0], sizeof(float4) * (size_t)b.N, cudaMemcpyDeviceToDevice, st);
  // solveA(k) records the scenes' largest solid displacement in slot k & 1
  // (the reorder cleared both), solveB(k) clears the other for iteration k+1
  int in = 0;
  // an early-stopped active-set solve captured into a graph runs its last
  // iterations (from the first after which no PBF pass follows) as a device
  // loop; elsewhere every iteration is enqueued (those past a scene's stop
  // find nothing to do)
  int kLoop = sch.K;
  cudaStreamCaptureStatus capSt = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &capSt);
  if (sch.active && capSt == cudaStreamCaptureStatusActive) {
    int k0 = sch.K;
    while (k0 - 1 >= 2 && !sch.pbf[k0 - 1]) --k0;
    if (sch.K - k0 >= 2) kLoop = k0;
  }
  for (int k = 0; k < kLoop; ++k) {
    // iteration 0 after computeL with features: it already evaluated the
    // constraint at these velocities, with one lane per slot (several lanes
    // sum in another order, so they evaluate it again)
    const int stored = k == 0 && sch.features && sch.lanes == 1 ? kStoredC : 0;
    // active set: iteration 0 visits every slot and marks what moved; later
    // ones visit the marked slots; velocities update in place (solveB and
    // pbfB read no neighbour's velocity), so there is no ping-pong
    // iteration 0 moves every particle, so iteration 1 visits every one
    // (skipping from it would only add the marking); it marks what it moves
    // for iteration 2, from which on only marked particles are visited
    const int act = sch.active ? (kInPlace | (k >= 1 ? kMarkMoved : 0) | (k >= 2 ? kActive : 0)) : 0;
    if (sch.active && k >= 2) {
      // solveA and solveB run over compacted lists of the slots they visit
      // (full warps however the slots are spread); velocities stay in
      // velS[0] (in place from iteration 0 on). Before a PBF pass every
      // slot's predicted position is brought up to date, as the per-slot
      // solveB would have left it.
      enqueueListIteration(b, sch, k, aflags, st, R);
      if (sch.pbf[k]) {
        launch_predict(b, b.velS[0], st);
        R.mark(st, "predict");
      }
    } else {
      launch_solveA(b, k, b.velS[in], aflags | stored | (act & kActive), sch.varA, sch.lanes, st);
      R.mark(st, "solveA");
      launch_solveB(b, k, b.velS[in], b.velS[in ^ (sch.active ? 0 : 1)], sch.pbf[k] != 0,
                    (sch.reduce ? kTrackResid : 0) | act, sch.varB, sch.lanes, st);
      R.mark(st, "solveB");
      if (sch.reduce) {
        launch_resid_reduce(b, k, (aflags & kWarm) != 0, st);
        R.mark(st, "residual");
      }
    }
    if (!sch.active) in ^= 1;
    if (sch.pbf[k]) {
      launch_pbfA(b, k, b.velS[in], 0, st);
      R.mark(st, "pbfA");
      launch_pbfB(b, k, b.velS[in], b.velS[in ^ (sch.active ? 0 : 1)],
                  sch.active ? (kInPlace | (k >= 1 ? kMarkMoved : 0)) : 0, st);
      R.mark(st, "pbfB");
      if (!sch.active) in ^= 1;
    }
  }
  if (kLoop < sch.K) {
    const cudaError_t e = captureDeviceLoop(s, sch, kLoop, aflags, st);
    if (e != cudaSuccess) return e;
  }
  if (sch.fallback) {
    // the judge: scenes that did not stop within their cap are re-solved
    // with the reference solve from vel0 (in a graph, behind a conditional
    // node that skips the body when every scene stopped)
    if (capSt == cudaStreamCaptureStatusActive) {
      const cudaError_t e = captureFallback(s, sch, in, st);
      if (e != cudaSuccess) return e;
    } else {
      launch_judge(b, 0, false, st);
      R.mark(st, "judge");
      enqueuePlainResolve(s, sch, in, st, R);
    }
  }
  if (sch.track) {  // residual of the state the iterations leave behind
    launch_solveA(b, sch.K, b.velS[in], kTrackResid | kMeasureOnly, sch.varA, sch.lanes, st);
    R.mark(st, "solveA(measure)");
    launch_solveB(b, sch.K, b.velS[in], nullptr, false, kTrackResid | kMeasureOnly, sch.varB, sch.lanes, st);
    R.mark(st, "solveB(measure)");
    launch_resid_reduce(b, -1, false, st);
    R.mark(st, "residual");
  }
  launch_xsph(b, b.velS[in], b.velS[in ^ 1], st);
  R.mark(st, "xsph");
  in ^= 1;
  // the update moves the particles: asynchronous read-backs of the previous
  // positions (xpbi_read_positions_async) must have finished (inside a
  // captured graph, as an external event wait node)
  {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cs);
    cudaStreamWaitEvent(st, s->evCopy, cs == cudaStreamCaptureStatusActive ? cudaEventWaitExternal : 0);
  }
  launch_updateF_integrate(b, b.velS[in], st);
  R.mark(st, "updateF+integrate");
  if (sch.keepLam) {
    launch_keep_lambda(b, st);
    R.mark(st, "keepLambda");
  }
  return cudaSuccess;
}

int kernelsPerSubstep(const Schedule& sch) {
  int n = 5 /* count, scan, fill, bigcells, reorder */ + 1 /* computeL */ + 2 /* xsph, updateF+integrate */;
  for (int k = 0; k < sch.K; ++k) {
    const bool list = sch.active && k >= 2;  // two compactions; before a PBF pass, the predicted positions
    n += 2 + (sch.pbf[k] ? 2 : 0) + (sch.reduce ? 1 : 0) + (list ? 2 + (sch.pbf[k] ? 1 : 0) : 0);
  }
  if (sch.mode == 1) n += 2;
  if (sch.mode == 2) n += 1;
  if (sch.track) n += 3;
  if (sch.keepLam) n += 1;
  if (sch.fallback) n += 1;  // the judge (its plain re-solve launches only when a scene failed)
  return n;
}

int createImpl(const xpbi_scene_desc* scenes, uint32_t nScenes, xpbi_sim** out) {
  if (!out) return fail(XPBI_ERR_INVALID, "out handle pointer is NULL");
  *out = nullptr;
  if (nScenes < 1 || nScenes > 65535) return fail(XPBI_ERR_INVALID, "n_scenes must be 1..65535");
  std::vector<SceneHost> sc(nScenes);
  uint64_t N = 0, C = 0;
  for (uint32_t i = 0; i < nScenes; ++i) {
    XPBI_TRY(validateScene(&scenes[i]));
    SceneHost& h = sc[i];
    XPBI_TRY(sizeGrid(scenes[i], h));
    h.n = scenes[i].n;
    h.pBase = (uint32_t)N;
    h.cellBase = (uint32_t)C;
    h.nMats = scenes[i].n_materials;
    std::memset(h.mats, 0, sizeof(h.mats));
    for (uint32_t m = 0; m < h.nMats; ++m) h.mats[m] = scenes[i].materials[m];
    for (uint32_t k = 0; k < h.n; ++k) ++h.matCount[scenes[i].mat_ids[k]];
    defaultParams(h, h.params);
    N += h.n;
    C += h.numCells;
  }
  if (N >= 0x7fffffffull) return fail(XPBI_ERR_INVALID, "too many particles");
  if (C >= 0x7fffffffull) return fail(XPBI_ERR_INVALID, "too many cells");
  xpbi_sim* s = new xpbi_sim();
  s->sc = std::move(sc);
  int rc = XPBI_OK;
  auto bail = [&](int code) {
    destroyAll(s);
    delete s;
    return code;
  };
  if (cudaGetDevice(&s->device) != cudaSuccess) return bail(fail(XPBI_ERR_CUDA, "no CUDA device"));
  if (cudaStreamCreateWithFlags(&s->own, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->capture, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->loop, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->evWork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->evCopy, cudaEventDisableTiming) != cudaSuccess)
    return bail(fail(XPBI_ERR_CUDA, "cudaStreamCreate failed"));
  s->stream = s->own;
  Bufs& b = s->b;
  b.N = (uint32_t)N;
  b.C = (uint32_t)C;
  b.S = nScenes;
  b.maxSceneN = 0;
  for (const SceneHost& h : s->sc) b.maxSceneN = std::max<uint32_t>(b.maxSceneN, (uint32_t)h.n);
  b.scanTiles = scan_tiles(b.C);
  const size_t n = std::max<size_t>(b.N, 1);
#define A(ptr, cnt)                               \
  do {                                            \
    rc = alloc(s, &(ptr), (cnt));                 \
    if (rc != XPBI_OK) return bail(rc);           \
  } while (0)
  A(b.pos, n);
  A(b.vel, n);
  A(b.F, 9 * n);
  A(b.state, n);
  A(b.posS, n);
  A(b.velS[0], n);
  A(b.velS[1], n);
  A(b.FS, 9 * n);
  A(b.stateS, n);
  A(b.L, 9 * n);
  A(b.sgP, 3 * n);
  A(b.lam, n);
  A(b.pbfLam, n);
  A(b.Sp, 4 * n);
  A(b.SpSelf, n);
  A(b.key, n);
  A(b.tmp, n);
  A(b.sortedIdx, n);
  A(b.cursor, (size_t)b.C + 4);
  A(b.cellStart, (size_t)b.C + 4);
  A(b.cellWater, (size_t)b.C + 16);
  unsigned long long* ctl = nullptr;
  A(ctl, (size_t)b.scanTiles + 1);
  b.tileTicket = reinterpret_cast<uint32_t*>(ctl);
  b.bigCount = reinterpret_cast<uint32_t*>(ctl) + 1;
  b.tileStatus = ctl + 1;
  A(b.bigList, n / 64 + 2);
  A(b.sceneOf, n);
  A(b.nbr, (size_t)kNbrCap * n);
  A(b.nbrCount, n);
  A(b.nbrP, (size_t)kNbrCap * n);
  A(b.nbrPCount, n);
  A(b.xc, n);
  A(b.pbfRec, n);
  A(b.lamOut, n);
  A(b.lamPrev, n);
  A(b.lamWarm, n);
  A(b.feat, (size_t)kFeat * n);
  A(b.cons0, 4 * n);
  A(b.netOut, n);
  A(b.rr, n);
  A(b.c0sq, n);
  A(b.rc, n);
  A(b.solidDisp, 2 * (size_t)nScenes);
  A(b.residPart, (size_t)nScenes * kResidBlocks * 4);
  A(b.residTicket, nScenes);
  A(b.resid, (size_t)nScenes * kMaxResid);
  A(b.residC, (size_t)nScenes * kMaxResid);
  A(b.c0, nScenes);
  A(b.cc0, nScenes);
  A(b.done, nScenes);
  // flag arrays padded to whole 16-byte groups (the compaction reads 16 at once)
  A(b.dirty[0], (n + 15) & ~size_t(15));
  A(b.dirty[1], (n + 15) & ~size_t(15));
  A(b.bmark, (n + 15) & ~size_t(15));
  A(b.imp, n);
  A(b.listA, n);
  A(b.listB, n);
  A(b.thr, 3 * (size_t)nScenes);
  A(b.dv0sq, n);
  A(b.actA, (size_t)kMaxResid);
  A(b.actB, (size_t)kMaxResid);
  A(b.kIter, 1);
  A(b.vel0, n);
  A(b.rerun, nScenes);
  A(b.itersUsed, nScenes);
  {
    uint8_t* blob = nullptr;
    A(blob, mlp_blob_bytes());
    b.netBlob = blob;
  }
  A(s->netParams, 9473);
  A(s->netErr, 1);
  A(b.scenes, nScenes);
  A(b.mats, (size_t)nScenes * kMaxMats);
  A(b.err, 1);
  A(b.waitProbe, 1);
  A(s->matWords, (size_t)nScenes * kMaxMats * XPBI_MATERIAL_WORDS);
#undef A
  // initial state (sim.js:52-81)
  std::vector<float4> pos(n), vel(n);
  std::vector<float> F(9 * n, 0.f), state(n, 0.f), zero(n, 0.f);
  std::vector<uint16_t> sceneOf(n, 0);
  for (uint32_t si = 0; si < nScenes; ++si) {
    const xpbi_scene_desc& d = scenes[si];
    const SceneHost& h = s->sc[si];
    for (uint32_t k = 0; k < d.n; ++k) {
      const size_t i = h.pBase + k;
      const float seed = d.color_seeds ? d.color_seeds[k] : 0.f;
      pos[i] = make_float4(d.positions[3 * k], d.positions[3 * k + 1], d.positions[3 * k + 2],
                           (float)d.mat_ids[k] + seed);
      vel[i] = d.velocities ? make_float4(d.velocities[3 * k], d.velocities[3 * k + 1], d.velocities[3 * k + 2], 0.f)
                            : make_float4(0.f, 0.f, 0.f, 0.f);
      state[i] = d.states ? d.states[k] : 0.f;
      sceneOf[i] = (uint16_t)si;
    }
  }
  for (size_t i = 0; i < b.N; ++i) {
    F[0 * n + i] = 1.f;  // plane (c=0,r=0)
    F[4 * n + i] = 1.f;  // plane (c=1,r=1)
    F[8 * n + i] = 1.f;  // plane (c=2,r=2)
  }
  auto H2D = [&](void* dst, const void* src, size_t bytes) {
    return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  };
  bool ok = H2D(b.pos, pos.data(), 16 * n) && H2D(b.vel, vel.data(), 16 * n) && H2D(b.F, F.data(), 36 * n) &&
            H2D(b.state, state.data(), 4 * n) && H2D(b.lam, zero.data(), 4 * n) &&
            H2D(b.pbfLam, zero.data(), 4 * n) && H2D(b.sceneOf, sceneOf.data(), 2 * n) &&
            cudaMemset(b.err, 0, sizeof(int)) == cudaSuccess &&
            cudaMemset(b.waitProbe, 0, sizeof(unsigned long long)) == cudaSuccess && cudaMemset(b.L, 0, 36 * n) == cudaSuccess &&
            cudaMemset(b.sortedIdx, 0, 4 * n) == cudaSuccess && cudaMemset(b.lamOut, 0, 4 * n) == cudaSuccess &&
            cudaMemset(b.lamPrev, 0, 4 * n) == cudaSuccess && cudaMemset(b.lamWarm, 0, 4 * n) == cudaSuccess &&
            cudaMemset(b.done, 0, sizeof(int) * nScenes) == cudaSuccess &&
            cudaMemset(b.actA, 0, sizeof(uint32_t) * kMaxResid) == cudaSuccess &&
            cudaMemset(b.rerun, 0, sizeof(int) * nScenes) == cudaSuccess &&
            cudaMemset(b.actB, 0, sizeof(uint32_t) * kMaxResid) == cudaSuccess &&
            cudaMemset(b.itersUsed, 0, sizeof(int) * nScenes) == cudaSuccess &&
            cudaMemset(b.resid, 0, sizeof(double) * nScenes * kMaxResid) == cudaSuccess &&
            cudaMemset(b.residC, 0, sizeof(double) * nScenes * kMaxResid) == cudaSuccess &&
            cudaMemset(b.cc0, 0, sizeof(double) * nScenes) == cudaSuccess &&
            cudaMemset(b.residTicket, 0, sizeof(uint32_t) * nScenes) == cudaSuccess &&
            cudaMemset(s->netErr, 0, sizeof(int)) == cudaSuccess &&
            cudaMemset(b.cellStart, 0, 4 * ((size_t)b.C + 4)) == cudaSuccess;
  if (!ok) return bail(fail(XPBI_ERR_CUDA, "initial upload failed"));
  // sets the network kernel's shared-memory attribute outside any capture
  if (mlp_forward(nullptr, 0, nullptr, nullptr, nullptr, nullptr, s->stream) != cudaSuccess)
    return bail(fail(XPBI_ERR_CUDA, "network kernel attribute"));
  rc = upload(s);
  if (rc != XPBI_OK) return bail(rc);
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return bail(fail(XPBI_ERR_CUDA, "initial sync failed"));
  *out = s;
  return XPBI_OK;
}

int checkSim(const xpbi_sim* s) {
  if (!s) return fail(XPBI_ERR_INVALID, "sim handle is NULL");
  return XPBI_OK;
}

int applySchedule(xpbi_sim* s, int32_t iterations, int32_t hasWater) {
  if (iterations >= 0) {
    if (iterations > 100000) return fail(XPBI_ERR_INVALID, "iterations out of range");
    for (SceneHost& h : s->sc) {
      if (h.iterations != iterations || h.hasWater != (hasWater ? 1 : 0)) s->dirty = true;
      h.iterations = iterations;
      h.hasWater = hasWater ? 1 : 0;
    }
  }
  return XPBI_OK;
}

int checkDeviceErr(xpbi_sim* s) {
  int e = 0, en = 0;
  XPBI_CK(cudaMemcpyAsync(&e, s->b.err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  XPBI_CK(cudaMemcpyAsync(&en, s->netErr, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  XPBI_CK(cudaStreamSynchronize(s->stream));
  e |= en;
  if (e) {
    cudaMemsetAsync(s->b.err, 0, sizeof(int), s->stream);
    cudaMemsetAsync(s->netErr, 0, sizeof(int), s->stream);
    cudaStreamSynchronize(s->stream);
    char msg[96];
    std::snprintf(msg, sizeof(msg), "device error word 0x%x (bounded wait expired in the prefix scan)", e);
    return fail(XPBI_ERR_DEVICE, msg);
  }
  return XPBI_OK;
}

int ensureGraph(xpbi_sim* s, const Schedule& sch) {
  const std::string key = sch.key();
  if (s->gexec && key == s->gkey) return XPBI_OK;
  if (s->gexec) {
    cudaGraphExecDestroy(s->gexec);
    s->gexec = nullptr;
  }
  if (s->graph) {
    cudaGraphDestroy(s->graph);
    s->graph = nullptr;
  }
  XPBI_CK(cudaStreamBeginCapture(s->capture, cudaStreamCaptureModeThreadLocal));
  const cudaError_t qe = enqueueSubstep(s, sch, s->capture, nullptr);
  cudaGraph_t g = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(s->capture, &g);  // ends the capture whatever happened
  if (qe != cudaSuccess || ee != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return fail(XPBI_ERR_CUDA, std::string("substep graph capture: ") +
                                   cudaGetErrorString(qe != cudaSuccess ? qe : ee));
  }
  s->graph = g;
  XPBI_CK(cudaGraphInstantiate(&s->gexec, g, 0));
  s->gkey = key;
  return XPBI_OK;
}

}  // namespace

extern "C" {

const char* xpbi_last_error(void) { return g_err.c_str(); }

int xpbi_pack_uniforms(const xpbi_scene_desc* scene, const xpbi_params* params,
                       uint32_t params_words[XPBI_PARAMS_WORDS],
                       uint32_t material_words[XPBI_MAX_MATERIALS * XPBI_MATERIAL_WORDS]) {
  XPBI_TRY(validateScene(scene));
  if (!params_words || !material_words) return fail(XPBI_ERR_INVALID, "output words are NULL");
  SceneHost h;
  XPBI_TRY(sizeGrid(*scene, h));
  h.n = scene->n;
  if (params) h.params = *params;
  else std::memset(&h.params, 0, sizeof(h.params));
  packParams(h, h.params, params_words);
  std::memset(material_words, 0, 4 * XPBI_MAX_MATERIALS * XPBI_MATERIAL_WORDS);
  for (uint32_t m = 0; m < scene->n_materials; ++m) packMaterial(scene->materials[m], h.V0, material_words + 16 * m);
  return XPBI_OK;
}

int xpbi_create(const xpbi_scene_desc* scene, xpbi_sim** out) { return createImpl(scene, 1, out); }

int xpbi_batch_create(const xpbi_scene_desc* scenes, uint32_t n_scenes, xpbi_sim** out) {
  if (!scenes) return fail(XPBI_ERR_INVALID, "scenes is NULL");
  return createImpl(scenes, n_scenes, out);
}

void xpbi_destroy(xpbi_sim* sim) {
  if (!sim) return;
  cudaStreamSynchronize(sim->stream);
  if (sim->copy) cudaStreamSynchronize(sim->copy);
  destroyAll(sim);
  delete sim;
}

int xpbi_write_materials(xpbi_sim* sim, int32_t scene, const xpbi_material* materials, uint32_t n) {
  XPBI_TRY(checkSim(sim));
  if (!materials || n < 1 || n > (uint32_t)kMaxMats) return fail(XPBI_ERR_INVALID, "materials must be 1..8");
  for (uint32_t i = 0; i < n; ++i)
    if (materials[i].kind > XPBI_WATER) return fail(XPBI_ERR_INVALID, "material kind out of range");
  if (scene >= (int32_t)sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  for (uint32_t s = 0; s < sim->sc.size(); ++s) {
    if (scene >= 0 && (uint32_t)scene != s) continue;
    if (n < sim->sc[s].nMats) return fail(XPBI_ERR_INVALID, "fewer materials than the scene references");
    for (uint32_t m = 0; m < n; ++m) sim->sc[s].mats[m] = materials[m];
    sim->sc[s].nMats = n;
  }
  sim->dirty = true;
  return XPBI_OK;
}

int xpbi_write_params(xpbi_sim* sim, int32_t scene, const xpbi_params* params) {
  XPBI_TRY(checkSim(sim));
  if (!params) return fail(XPBI_ERR_INVALID, "params is NULL");
  if (!(params->dt > 0.f) || !std::isfinite(params->dt)) return fail(XPBI_ERR_INVALID, "dt must be positive");
  if (scene >= (int32_t)sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  for (uint32_t s = 0; s < sim->sc.size(); ++s) {
    if (scene >= 0 && (uint32_t)scene != s) continue;
    sim->sc[s].params = *params;
  }
  sim->dirty = true;
  return XPBI_OK;
}

int xpbi_set_schedule(xpbi_sim* sim, int32_t scene, int32_t iterations, int32_t has_water) {
  XPBI_TRY(checkSim(sim));
  if (iterations < 0 || iterations > 100000) return fail(XPBI_ERR_INVALID, "iterations out of range");
  if (scene >= (int32_t)sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  for (uint32_t s = 0; s < sim->sc.size(); ++s) {
    if (scene >= 0 && (uint32_t)scene != s) continue;
    sim->sc[s].iterations = iterations;
    sim->sc[s].hasWater = has_water ? 1 : 0;
  }
  sim->dirty = true;
  return XPBI_OK;
}

int xpbi_encode_substep(xpbi_sim* sim, int32_t iterations, int32_t has_water) {
  XPBI_TRY(checkSim(sim));
  for (const SceneHost& h : sim->sc)
    if (!(h.params.dt > 0.f)) return fail(XPBI_ERR_INVALID, "write_params must be called before stepping");
  XPBI_TRY(applySchedule(sim, iterations, has_water));
  XPBI_TRY(upload(sim));
  if (sim->b.N == 0) return XPBI_OK;
  XPBI_CK(enqueueSubstep(sim, schedule(sim), sim->stream, nullptr));
  XPBI_CK(cudaGetLastError());
  sim->fresh = false;
  sim->waterLPending = true;
  return XPBI_OK;
}

int xpbi_step(xpbi_sim* sim, int32_t substeps, int32_t iterations, int32_t has_water) {
  XPBI_TRY(checkSim(sim));
  if (substeps < 0) return fail(XPBI_ERR_INVALID, "substeps must be >= 0");
  for (const SceneHost& h : sim->sc)
    if (!(h.params.dt > 0.f)) return fail(XPBI_ERR_INVALID, "write_params must be called before stepping");
  XPBI_TRY(applySchedule(sim, iterations, has_water));
  XPBI_TRY(upload(sim));
  if (sim->b.N == 0 || substeps == 0) return XPBI_OK;
  XPBI_TRY(ensureGraph(sim, schedule(sim)));
  for (int i = 0; i < substeps; ++i) XPBI_CK(cudaGraphLaunch(sim->gexec, sim->stream));
  sim->fresh = false;
  sim->waterLPending = true;
  return XPBI_OK;
}

int xpbi_synchronize(xpbi_sim* sim) {
  XPBI_TRY(checkSim(sim));
  XPBI_CK(cudaStreamSynchronize(sim->stream));
  if (sim->copy) XPBI_CK(cudaStreamSynchronize(sim->copy));
  sim->copyPending = false;
  return checkDeviceErr(sim);
}

int xpbi_set_stream(xpbi_sim* sim, void* cuda_stream) {
  XPBI_TRY(checkSim(sim));
  XPBI_TRY(xpbi_synchronize(sim));
  sim->stream = cuda_stream ? (cudaStream_t)cuda_stream : sim->own;
  return XPBI_OK;
}

int xpbi_read_state(xpbi_sim* sim, uint32_t scene, float* pos4, float* vel4, float* F12, float* L12, float* aux4,
                    uint32_t* sorted_idx, uint32_t* cell_tab) {
  XPBI_TRY(checkSim(sim));
  if (scene >= sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  if (L12 && sim->waterLPending && sim->b.N > 0) {
    launch_computeL_water(sim->b, sim->stream);
    XPBI_CK(cudaGetLastError());
    sim->waterLPending = false;
  }
  XPBI_TRY(xpbi_synchronize(sim));
  const SceneHost& h = sim->sc[scene];
  const Bufs& b = sim->b;
  const size_t n = h.n, o = h.pBase, N = b.N;
  if (n == 0) {
    if (cell_tab) XPBI_CK(cudaMemcpy(cell_tab, b.cellStart + h.cellBase, 4 * (size_t)h.numCells, cudaMemcpyDeviceToHost));
    return XPBI_OK;
  }
  std::vector<float4> v(n);
  if (pos4) XPBI_CK(cudaMemcpy(pos4, b.pos + o, 16 * n, cudaMemcpyDeviceToHost));
  XPBI_CK(cudaMemcpy(v.data(), b.vel + o, 16 * n, cudaMemcpyDeviceToHost));
  if (vel4) std::memcpy(vel4, v.data(), 16 * n);
  auto planes = [&](const float* src, float* dst12) -> int {
    std::vector<float> t(9 * n);
    for (int p = 0; p < 9; ++p)
      XPBI_CK(cudaMemcpy(t.data() + p * n, src + p * N + o, 4 * n, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i)
      for (int c = 0; c < 3; ++c) {
        for (int r = 0; r < 3; ++r) dst12[12 * i + 4 * c + r] = t[(3 * c + r) * n + i];
        dst12[12 * i + 4 * c + 3] = 0.f;
      }
    return XPBI_OK;
  };
  if (F12) XPBI_TRY(planes(b.F, F12));
  if (L12) XPBI_TRY(planes(b.L, L12));
  if (aux4) {
    std::vector<float> lam(n), st(n), pl(n);
    XPBI_CK(cudaMemcpy(lam.data(), b.lam + o, 4 * n, cudaMemcpyDeviceToHost));
    XPBI_CK(cudaMemcpy(st.data(), b.state + o, 4 * n, cudaMemcpyDeviceToHost));
    XPBI_CK(cudaMemcpy(pl.data(), b.pbfLam + o, 4 * n, cudaMemcpyDeviceToHost));
    const float V0 = (float)h.V0;
    for (size_t i = 0; i < n; ++i) {
      aux4[4 * i] = sim->fresh ? V0 : v[i].w;  // aux.x = V^n (== vel.w after a substep)
      aux4[4 * i + 1] = lam[i];
      aux4[4 * i + 2] = st[i];
      aux4[4 * i + 3] = pl[i];
    }
  }
  if (sorted_idx) {
    XPBI_CK(cudaMemcpy(sorted_idx, b.sortedIdx + o, 4 * n, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i) sorted_idx[i] -= (uint32_t)o;
  }
  if (cell_tab) {
    XPBI_CK(cudaMemcpy(cell_tab, b.cellStart + h.cellBase, 4 * (size_t)h.numCells, cudaMemcpyDeviceToHost));
    for (size_t c = 0; c < h.numCells; ++c) cell_tab[c] -= (uint32_t)o;
  }
  return XPBI_OK;
}

int xpbi_read_positions(xpbi_sim* sim, uint32_t scene, float* out_pos4) {
  XPBI_TRY(checkSim(sim));
  if (!out_pos4) return fail(XPBI_ERR_INVALID, "output is NULL");
  if (scene >= sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  const SceneHost& h = sim->sc[scene];
  if (h.n == 0) return XPBI_OK;
  XPBI_CK(cudaMemcpyAsync(out_pos4, sim->b.pos + h.pBase, 16 * (size_t)h.n, cudaMemcpyDeviceToHost, sim->stream));
  return xpbi_synchronize(sim);
}

int xpbi_read_positions_async(xpbi_sim* sim, uint32_t scene, float* out_pos4) {
  XPBI_TRY(checkSim(sim));
  if (!out_pos4) return fail(XPBI_ERR_INVALID, "output is NULL");
  if (scene >= sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  const SceneHost& h = sim->sc[scene];
  if (h.n == 0) return XPBI_OK;
  XPBI_CK(cudaEventRecord(sim->evWork, sim->stream));
  XPBI_CK(cudaStreamWaitEvent(sim->copy, sim->evWork, 0));
  XPBI_CK(cudaMemcpyAsync(out_pos4, sim->b.pos + h.pBase, 16 * (size_t)h.n, cudaMemcpyDeviceToHost, sim->copy));
  XPBI_CK(cudaEventRecord(sim->evCopy, sim->copy));
  sim->copyPending = true;
  return XPBI_OK;
}

int xpbi_read_velocities(xpbi_sim* sim, uint32_t scene, float* out_vel4) {
  XPBI_TRY(checkSim(sim));
  if (!out_vel4) return fail(XPBI_ERR_INVALID, "output is NULL");
  if (scene >= sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  const SceneHost& h = sim->sc[scene];
  if (h.n == 0) return XPBI_OK;
  XPBI_CK(cudaMemcpyAsync(out_vel4, sim->b.vel + h.pBase, 16 * (size_t)h.n, cudaMemcpyDeviceToHost, sim->stream));
  return xpbi_synchronize(sim);
}

int xpbi_write_state(xpbi_sim* sim, uint32_t scene, const float* pos4, const float* vel4, const float* F12,
                     const float* aux4) {
  XPBI_TRY(checkSim(sim));
  XPBI_TRY(xpbi_synchronize(sim));  // read-backs in flight finish first
  if (scene >= sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  XPBI_CK(cudaStreamSynchronize(sim->stream));
  const SceneHost& h = sim->sc[scene];
  const Bufs& b = sim->b;
  const size_t n = h.n, o = h.pBase, N = b.N;
  if (n == 0) return XPBI_OK;
  if (pos4) {
    for (size_t i = 0; i < n; ++i) {
      float w = pos4[4 * i + 3];
      if (!(w >= 0.f) || (uint32_t)w >= h.nMats) return fail(XPBI_ERR_INVALID, "pos.w material index out of range");
    }
    XPBI_CK(cudaMemcpy(b.pos + o, pos4, 16 * n, cudaMemcpyHostToDevice));
  }
  if (vel4) XPBI_CK(cudaMemcpy(b.vel + o, vel4, 16 * n, cudaMemcpyHostToDevice));
  if (F12) {
    std::vector<float> t(n);
    for (int c = 0; c < 3; ++c)
      for (int r = 0; r < 3; ++r) {
        for (size_t i = 0; i < n; ++i) t[i] = F12[12 * i + 4 * c + r];
        XPBI_CK(cudaMemcpy(b.F + (3 * c + r) * N + o, t.data(), 4 * n, cudaMemcpyHostToDevice));
      }
  }
  if (aux4) {
    std::vector<float> lam(n), st(n), pl(n);
    for (size_t i = 0; i < n; ++i) {
      lam[i] = aux4[4 * i + 1];
      st[i] = aux4[4 * i + 2];
      pl[i] = aux4[4 * i + 3];
    }
    XPBI_CK(cudaMemcpy(b.lam + o, lam.data(), 4 * n, cudaMemcpyHostToDevice));
    XPBI_CK(cudaMemcpy(b.lamOut + o, lam.data(), 4 * n, cudaMemcpyHostToDevice));  // warm starts from it
    XPBI_CK(cudaMemcpy(b.state + o, st.data(), 4 * n, cudaMemcpyHostToDevice));
    XPBI_CK(cudaMemcpy(b.pbfLam + o, pl.data(), 4 * n, cudaMemcpyHostToDevice));
  }
  sim->fresh = false;
  return XPBI_OK;
}

int xpbi_read_uniforms(xpbi_sim* sim, uint32_t scene, uint32_t params_words[XPBI_PARAMS_WORDS],
                       uint32_t material_words[XPBI_MAX_MATERIALS * XPBI_MATERIAL_WORDS]) {
  XPBI_TRY(checkSim(sim));
  if (scene >= sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  const SceneHost& h = sim->sc[scene];
  if (params_words) packParams(h, h.params, params_words);
  if (material_words) {
    std::memset(material_words, 0, 4 * XPBI_MAX_MATERIALS * XPBI_MATERIAL_WORDS);
    for (uint32_t m = 0; m < h.nMats; ++m) packMaterial(h.mats[m], h.V0, material_words + 16 * m);
  }
  return XPBI_OK;
}

int xpbi_info(xpbi_sim* sim, uint32_t* n_particles, uint32_t* n_cells, uint32_t* n_scenes, int32_t dims[3]) {
  XPBI_TRY(checkSim(sim));
  if (n_particles) *n_particles = sim->b.N;
  if (n_cells) *n_cells = sim->b.C;
  if (n_scenes) *n_scenes = sim->b.S;
  if (dims)
    for (int k = 0; k < 3; ++k) dims[k] = sim->sc[0].dims[k];
  return XPBI_OK;
}

int xpbi_profile_substep(xpbi_sim* sim, int32_t iterations, int32_t has_water, float* ms, int32_t cap,
                         int32_t* count, char* labels, size_t labels_cap) {
  XPBI_TRY(checkSim(sim));
  drainCopies(sim);
  for (const SceneHost& h : sim->sc)
    if (!(h.params.dt > 0.f)) return fail(XPBI_ERR_INVALID, "write_params must be called before stepping");
  XPBI_TRY(applySchedule(sim, iterations, has_water));
  XPBI_TRY(upload(sim));
  if (sim->b.N == 0) {
    if (count) *count = 0;
    return XPBI_OK;
  }
  std::vector<cudaEvent_t> ev;
  std::vector<std::string> lab;
  Recorder rec;
  rec.ev = &ev;
  rec.labels = &lab;
  XPBI_CK(enqueueSubstep(sim, schedule(sim), sim->stream, &rec));
  XPBI_CK(cudaGetLastError());
  XPBI_CK(cudaStreamSynchronize(sim->stream));
  sim->fresh = false;
  sim->waterLPending = true;
  std::string text;
  const int nl = (int)lab.size();
  for (int k = 0; k < nl; ++k) {
    float t = 0.f;
    cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
    if (ms && k < cap) ms[k] = t;
    char line[96];
    std::snprintf(line, sizeof(line), "%s: %.3fms\n", lab[k].c_str(), t);
    text += line;
  }
  for (cudaEvent_t e : ev) cudaEventDestroy(e);
  if (count) *count = nl;
  if (labels && labels_cap > 0) {
    size_t m = std::min(labels_cap - 1, text.size());
    std::memcpy(labels, text.data(), m);
    labels[m] = 0;
  }
  return checkDeviceErr(sim);
}

int xpbi_autotune(xpbi_sim* sim, int32_t iterations, int32_t has_water, int32_t repeats, int32_t* chosen,
                  float* ms, int32_t cap) {
  XPBI_TRY(checkSim(sim));
  drainCopies(sim);
  for (const SceneHost& h : sim->sc)
    if (!(h.params.dt > 0.f)) return fail(XPBI_ERR_INVALID, "write_params must be called before xpbi_autotune");
  if (repeats < 1 || repeats > 1000) return fail(XPBI_ERR_INVALID, "repeats must be 1..1000");
  XPBI_TRY(applySchedule(sim, iterations, has_water));
  XPBI_TRY(upload(sim));
  const Bufs& b = sim->b;
  cudaStream_t st = sim->stream;
  float t[kSolveAVariants + kSolveBVariants] = {0.f};
  if (b.N > 0) {
    // what read_state reports of the last substep and the timing runs
    // overwrite (sort outputs, Bonet-Lok correction, multipliers): keep it
    struct Saved {
      void* dev;
      size_t bytes;
    };
    const Saved keep[] = {{b.sortedIdx, 4 * (size_t)b.N},
                          {b.cellStart, 4 * ((size_t)b.C + 1)},
                          {b.L, 36 * (size_t)b.N},
                          {b.lam, 4 * (size_t)b.N}};
    size_t total = 0;
    for (const Saved& k : keep) total += (k.bytes + 255) & ~(size_t)255;
    uint8_t* save = nullptr;
    if (cudaMalloc(&save, total) != cudaSuccess) return fail(XPBI_ERR_OOM, "xpbi_autotune scratch");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto timed = [&](auto&& launch) {
      launch();  // warm-up
      cudaEventRecord(e0, st);
      for (int r = 0; r < repeats; ++r) launch();
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float x = 0.f;
      cudaEventElapsedTime(&x, e0, e1);
      return x / repeats;
    };
    {
      size_t off = 0;
      for (const Saved& k : keep) {
        cudaMemcpyAsync(save + off, k.dev, k.bytes, cudaMemcpyDeviceToDevice, st);
        off += (k.bytes + 255) & ~(size_t)255;
      }
    }
    // the substep's preparation on the current state; it writes only the
    // substep's working buffers, which the next substep rewrites
    launch_count(b, st);
    launch_scan(b, st);
    launch_scatter(b, st);
    launch_reorder(b, false, st);
    launch_computeL(b, true, false, st);
    cudaMemsetAsync(b.done, 0, sizeof(int) * b.S, st);  // no scene counts as converged here
    cudaMemsetAsync(b.solidDisp, 0, sizeof(uint32_t) * 2 * b.S, st);
    // iteration 0 of each variant from lambda = 0, then solveB on its record
    for (int v = 0; v < kSolveAVariants; ++v)
      t[v] = timed([&] { launch_solveA(b, 0, b.velS[0], 0, v, 1, st); });
    int bestA = 0;
    for (int v = 1; v < kSolveAVariants; ++v)
      if (t[v] < t[bestA]) bestA = v;
    if (t[0] <= 1.01f * t[bestA]) bestA = 0;  // keep the default on a near tie
    launch_solveA(b, 0, b.velS[0], 0, bestA, 1, st);
    for (int v = 0; v < kSolveBVariants; ++v)
      t[kSolveAVariants + v] = timed([&] { launch_solveB(b, 0, b.velS[0], b.velS[1], false, 0, v, 1, st); });
    int bestB = 0;
    for (int v = 1; v < kSolveBVariants; ++v)
      if (t[kSolveAVariants + v] < t[kSolveAVariants + bestB]) bestB = v;
    if (t[kSolveAVariants] <= 1.01f * t[kSolveAVariants + bestB]) bestB = 0;
    {
      size_t off = 0;
      for (const Saved& k : keep) {
        cudaMemcpyAsync(k.dev, save + off, k.bytes, cudaMemcpyDeviceToDevice, st);
        off += (k.bytes + 255) & ~(size_t)255;
      }
    }
    const cudaError_t e = cudaStreamSynchronize(st);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(save);
    if (e != cudaSuccess) return fail(XPBI_ERR_CUDA, std::string("xpbi_autotune: ") + cudaGetErrorString(e));
    XPBI_CK(cudaGetLastError());
    sim->tuneA = bestA;
    sim->tuneB = bestB;
  }
  if (chosen) {
    chosen[0] = sim->tuneA;
    chosen[1] = sim->tuneB;
  }
  for (int k = 0; k < cap && k < kSolveAVariants + kSolveBVariants; ++k)
    if (ms) ms[k] = t[k];
  return checkDeviceErr(sim);
}

int xpbi_set_lanes(xpbi_sim* sim, int32_t lanes) {
  XPBI_TRY(checkSim(sim));
  if (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4)
    return fail(XPBI_ERR_INVALID, "lanes must be 0 (by size), 1, 2 or 4");
  if (lanes > 1 && sim->b.N > (1u << 28)) return fail(XPBI_ERR_INVALID, "several lanes per slot need N <= 2^28");
  sim->lanesMode = lanes;
  return XPBI_OK;
}

int xpbi_set_variants(xpbi_sim* sim, int32_t solve_a, int32_t solve_b) {
  XPBI_TRY(checkSim(sim));
  if (solve_a >= kSolveAVariants || solve_b >= kSolveBVariants)
    return fail(XPBI_ERR_INVALID, "variant index out of range");
  if (solve_a >= 0) sim->tuneA = solve_a;
  if (solve_b >= 0) sim->tuneB = solve_b;
  return XPBI_OK;
}

namespace {
// main.js:33-62 in f64, stored as f32 like the reference's Float32Array
void lookAt(const double eye[3], const double tgt[3], float out[16]) {
  auto norm = [](double v[3]) {
    const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int k = 0; k < 3; ++k) v[k] /= l;
  };
  double z[3] = {eye[0] - tgt[0], eye[1] - tgt[1], eye[2] - tgt[2]};
  norm(z);
  const double up[3] = {0, 1, 0};
  double x[3] = {up[1] * z[2] - up[2] * z[1], up[2] * z[0] - up[0] * z[2], up[0] * z[1] - up[1] * z[0]};
  norm(x);
  const double y[3] = {z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]};
  auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
  const double m[16] = {x[0], y[0], z[0], 0, x[1], y[1], z[1], 0, x[2], y[2], z[2], 0,
                        -dot(x, eye), -dot(y, eye), -dot(z, eye), 1};
  for (int k = 0; k < 16; ++k) out[k] = (float)m[k];
}
void perspective(double fovY, double aspect, double nearZ, double farZ, float out[16]) {
  const double f = 1.0 / std::tan(fovY / 2);
  const double m[16] = {f / aspect, 0, 0, 0, 0, f, 0, 0, 0, 0, farZ / (nearZ - farZ), -1,
                        0, 0, (nearZ * farZ) / (nearZ - farZ), 0};
  for (int k = 0; k < 16; ++k) out[k] = (float)m[k];
}
void mul4(const float a[16], const float b[16], float out[16]) {  // a * b, column-major
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += (double)a[k * 4 + r] * (double)b[c * 4 + k];
      out[c * 4 + r] = (float)s;
    }
}
}  // namespace

int xpbi_render(xpbi_sim* sim, uint32_t scene, const xpbi_camera* cam, uint32_t width, uint32_t height,
                uint8_t* rgba_out, void** device_rgba) {
  XPBI_TRY(checkSim(sim));
  if (!cam) return fail(XPBI_ERR_INVALID, "camera is NULL");
  if (scene >= sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  if (width < 1 || height < 1 || width > 16384 || height > 16384)
    return fail(XPBI_ERR_INVALID, "image size must be 1..16384 per side");
  if (!(cam->fov_y > 0.f && cam->fov_y < 3.1f) || !(cam->near_z > 0.f && cam->far_z > cam->near_z))
    return fail(XPBI_ERR_INVALID, "camera needs 0 < fov_y < pi and 0 < near_z < far_z");
  XPBI_TRY(upload(sim));
  const SceneHost& h = sim->sc[scene];
  RenderParams P{};
  const double eye[3] = {cam->eye[0], cam->eye[1], cam->eye[2]};
  const double tgt[3] = {cam->target[0], cam->target[1], cam->target[2]};
  if (eye[0] == tgt[0] && eye[1] == tgt[1] && eye[2] == tgt[2]) return fail(XPBI_ERR_INVALID, "eye equals target");
  lookAt(eye, tgt, P.view);
  perspective(cam->fov_y, (double)width / height, cam->near_z, cam->far_z, P.proj);
  mul4(P.proj, P.view, P.viewProj);
  for (int k = 0; k < 3; ++k) {
    P.eye[k] = cam->eye[k];
    P.boxMin[k] = (float)h.dmin[k];
    P.boxMax[k] = (float)h.dmax[k];
  }
  const double l = std::sqrt((double)cam->light_dir[0] * cam->light_dir[0] +
                             (double)cam->light_dir[1] * cam->light_dir[1] +
                             (double)cam->light_dir[2] * cam->light_dir[2]);
  if (!(l > 0)) return fail(XPBI_ERR_INVALID, "light_dir must be nonzero");
  for (int k = 0; k < 3; ++k) P.lightDir[k] = (float)(cam->light_dir[k] / l);
  P.particleRadius = cam->particle_radius > 0.f ? cam->particle_radius : (float)(h.h * 0.62);
  P.groundY = (float)h.dmin[1];
  P.nearZ = cam->near_z;
  P.width = (int)width;
  P.height = (int)height;
  P.drawGround = cam->draw_ground ? 1 : 0;
  P.drawBox = cam->draw_box ? 1 : 0;
  P.maxPixelsPerParticle = 1 << 16;
  const size_t pixels = (size_t)width * height;
  if (pixels > sim->renderPixels) {
    if (sim->renderImg) cudaFree(sim->renderImg);
    if (sim->renderRgba) cudaFree(sim->renderRgba);
    sim->renderImg = nullptr;
    sim->renderRgba = nullptr;
    sim->renderPixels = 0;
    if (cudaMalloc(&sim->renderImg, 8 * pixels) != cudaSuccess ||
        cudaMalloc(&sim->renderRgba, 4 * pixels) != cudaSuccess)
      return fail(XPBI_ERR_OOM, "render target allocation failed");
    sim->renderPixels = pixels;
  }
  const Bufs& b = sim->b;
  render_frame(P, b.pos + h.pBase, b.vel + h.pBase, sim->matWords + (size_t)scene * kMaxMats * XPBI_MATERIAL_WORDS,
               h.n, sim->renderImg, sim->renderRgba, sim->stream);
  XPBI_CK(cudaGetLastError());
  if (rgba_out) {
    XPBI_CK(cudaMemcpyAsync(rgba_out, sim->renderRgba, 4 * pixels, cudaMemcpyDeviceToHost, sim->stream));
    XPBI_CK(cudaStreamSynchronize(sim->stream));
  }
  if (device_rgba) *device_rgba = sim->renderRgba;
  return checkDeviceErr(sim);
}

int xpbi_device_ptrs(xpbi_sim* sim, void** pos4, void** vel4, void** materials) {
  XPBI_TRY(checkSim(sim));
  if (pos4) *pos4 = sim->b.pos;
  if (vel4) *vel4 = sim->b.vel;
  if (materials) *materials = sim->matWords;
  return XPBI_OK;
}

int xpbi_set_solver(xpbi_sim* sim, int32_t mode, float rel_tol, float contact_rel_tol, int32_t track_residual,
                    int32_t log_features) {
  XPBI_TRY(checkSim(sim));
  if (mode < 0 || mode > 2) return fail(XPBI_ERR_INVALID, "solver mode must be 0, 1 or 2");
  if (mode == 1 && !sim->netLoaded) return fail(XPBI_ERR_INVALID, "network warm start needs xpbi_set_network first");
  if (!(rel_tol <= 1.f) || !std::isfinite(rel_tol)) return fail(XPBI_ERR_INVALID, "rel_tol must be <= 1");
  if (!(contact_rel_tol <= 1.f) || !std::isfinite(contact_rel_tol))
    return fail(XPBI_ERR_INVALID, "contact_rel_tol must be <= 1");
  sim->mode = mode;
  sim->residTol = rel_tol;
  sim->residTolC = contact_rel_tol < 0.f ? rel_tol : contact_rel_tol;
  sim->track = track_residual != 0;
  sim->features = log_features != 0;
  sim->dirty = true;
  return XPBI_OK;
}

int xpbi_set_active_set(xpbi_sim* sim, float share) {
  XPBI_TRY(checkSim(sim));
  if (!(share >= 0.f && share <= 1.f)) return fail(XPBI_ERR_INVALID, "active-set share must be in [0, 1]");
  sim->activeShare = share;
  sim->dirty = true;
  return XPBI_OK;
}

int xpbi_set_max_iterations(xpbi_sim* sim, int32_t max_iterations) {
  XPBI_TRY(checkSim(sim));
  if (max_iterations < 0 || max_iterations > kMaxResid - 1)
    return fail(XPBI_ERR_INVALID, "max_iterations must be 0.." + std::to_string(kMaxResid - 1));
  sim->maxIters = max_iterations;
  sim->dirty = true;
  return XPBI_OK;
}

int xpbi_read_fallback(xpbi_sim* sim, uint32_t scene, int32_t* resolved) {
  XPBI_TRY(checkSim(sim));
  if (scene >= sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  if (!resolved) return fail(XPBI_ERR_INVALID, "resolved is NULL");
  XPBI_TRY(xpbi_synchronize(sim));
  int r = 0;
  XPBI_CK(cudaMemcpy(&r, sim->b.rerun + scene, sizeof(int), cudaMemcpyDeviceToHost));
  *resolved = r;
  return XPBI_OK;
}

int xpbi_read_active_counts(xpbi_sim* sim, uint32_t* solve_a, uint32_t* solve_b, int32_t cap) {
  XPBI_TRY(checkSim(sim));
  if (cap < 0) return fail(XPBI_ERR_INVALID, "cap must be >= 0");
  XPBI_TRY(xpbi_synchronize(sim));
  const int m = std::min<int>(cap, kMaxResid);
  if (solve_a && m) XPBI_CK(cudaMemcpy(solve_a, sim->b.actA, sizeof(uint32_t) * m, cudaMemcpyDeviceToHost));
  if (solve_b && m) XPBI_CK(cudaMemcpy(solve_b, sim->b.actB, sizeof(uint32_t) * m, cudaMemcpyDeviceToHost));
  return XPBI_OK;
}

int xpbi_set_network(xpbi_sim* sim, const float* params, uint32_t count) {
  XPBI_TRY(checkSim(sim));
  if (!params || count != 9473u) return fail(XPBI_ERR_INVALID, "network needs 9473 parameters");
  XPBI_CK(cudaMemcpyAsync(sim->netParams, params, sizeof(float) * count, cudaMemcpyHostToDevice, sim->stream));
  mlp_pack(sim->netParams, sim->b.netBlob, sim->stream);
  XPBI_CK(cudaGetLastError());
  XPBI_CK(cudaStreamSynchronize(sim->stream));
  sim->netLoaded = true;
  return XPBI_OK;
}

int xpbi_read_residuals(xpbi_sim* sim, uint32_t scene, double* norms, int32_t cap, int32_t* iterations_run) {
  XPBI_TRY(checkSim(sim));
  if (scene >= sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  XPBI_TRY(xpbi_synchronize(sim));
  std::vector<double> r(kMaxResid);
  double c0 = 0;
  int used = 0;
  XPBI_CK(cudaMemcpy(r.data(), sim->b.resid + (size_t)scene * kMaxResid, sizeof(double) * kMaxResid,
                     cudaMemcpyDeviceToHost));
  XPBI_CK(cudaMemcpy(&c0, sim->b.c0 + scene, sizeof(double), cudaMemcpyDeviceToHost));
  XPBI_CK(cudaMemcpy(&used, sim->b.itersUsed + scene, sizeof(int), cudaMemcpyDeviceToHost));
  const int K = effIterations(sim, sim->sc[scene]);
  if (iterations_run) *iterations_run = used;
  if (norms && cap > 0) {
    // [ |C(v_pred)|, |r_0| .. |r_{K-1}|, |r| after the last applied iteration ]
    std::vector<double> out;
    out.push_back(std::sqrt(c0));
    for (int k = 0; k < K && k < kMaxResid - 1; ++k) out.push_back(k < used ? std::sqrt(r[k]) : NAN);
    out.push_back(std::sqrt(r[kMaxResid - 1]));
    for (int q = 0; q < cap && q < (int)out.size(); ++q) norms[q] = out[q];
  }
  return XPBI_OK;
}

int xpbi_read_contact_residuals(xpbi_sim* sim, uint32_t scene, double* norms, int32_t cap) {
  XPBI_TRY(checkSim(sim));
  if (scene >= sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  XPBI_TRY(xpbi_synchronize(sim));
  std::vector<double> r(kMaxResid);
  double c0 = 0;
  int used = 0;
  XPBI_CK(cudaMemcpy(r.data(), sim->b.residC + (size_t)scene * kMaxResid, sizeof(double) * kMaxResid,
                     cudaMemcpyDeviceToHost));
  XPBI_CK(cudaMemcpy(&c0, sim->b.cc0 + scene, sizeof(double), cudaMemcpyDeviceToHost));
  XPBI_CK(cudaMemcpy(&used, sim->b.itersUsed + scene, sizeof(int), cudaMemcpyDeviceToHost));
  const int K = effIterations(sim, sim->sc[scene]);
  if (norms && cap > 0) {
    // same slots as xpbi_read_residuals; slot 0 repeats iteration 0's value
    std::vector<double> out;
    out.push_back(std::sqrt(c0));
    for (int k = 0; k < K && k < kMaxResid - 1; ++k) out.push_back(k < used ? std::sqrt(r[k]) : NAN);
    out.push_back(std::sqrt(r[kMaxResid - 1]));
    for (int q = 0; q < cap && q < (int)out.size(); ++q) norms[q] = out[q];
  }
  return XPBI_OK;
}

int xpbi_read_particle_residuals(xpbi_sim* sim, uint32_t scene, float* r2, float* c2, float* r0sq) {
  XPBI_TRY(checkSim(sim));
  if (scene >= sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  XPBI_TRY(xpbi_synchronize(sim));
  const SceneHost& h = sim->sc[scene];
  const size_t n = h.n, o = h.pBase;
  if (n == 0) return XPBI_OK;
  if (r2) XPBI_CK(cudaMemcpy(r2, sim->b.rr + o, sizeof(float) * n, cudaMemcpyDeviceToHost));
  if (c2) XPBI_CK(cudaMemcpy(c2, sim->b.rc + o, sizeof(float) * n, cudaMemcpyDeviceToHost));
  if (r0sq) XPBI_CK(cudaMemcpy(r0sq, sim->b.c0sq + o, sizeof(float) * n, cudaMemcpyDeviceToHost));
  return XPBI_OK;
}

int xpbi_read_training(xpbi_sim* sim, uint32_t scene, float* features16, float* target, float* alpha_tilde) {
  XPBI_TRY(checkSim(sim));
  if (scene >= sim->sc.size()) return fail(XPBI_ERR_INVALID, "scene index out of range");
  XPBI_TRY(xpbi_synchronize(sim));
  const SceneHost& h = sim->sc[scene];
  const size_t n = h.n, o = h.pBase;
  if (features16) XPBI_CK(cudaMemcpy(features16, sim->b.feat + o * kFeat, sizeof(float) * kFeat * n,
                                      cudaMemcpyDeviceToHost));
  const float aT = sim->sdev[scene].alphaT;
  if (target) {
    XPBI_CK(cudaMemcpy(target, sim->b.lam + o, sizeof(float) * n, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i) target[i] *= aT;
  }
  if (alpha_tilde) *alpha_tilde = aT;
  return XPBI_OK;
}

int xpbi_test_wait_expiry(xpbi_sim* sim, uint32_t polls) {
  XPBI_TRY(checkSim(sim));
  if (polls < 1u || polls > (1u << 20)) return fail(XPBI_ERR_INVALID, "polls must be 1..1048576");
  launch_wait_expiry(sim->b, sim->b.waitProbe, polls, sim->stream);
  XPBI_CK(cudaGetLastError());
  return XPBI_OK;
}

int xpbi_launches_per_substep(xpbi_sim* sim, int32_t iterations, int32_t has_water, int32_t* out) {
  XPBI_TRY(checkSim(sim));
  if (!out) return fail(XPBI_ERR_INVALID, "out is NULL");
  XPBI_TRY(applySchedule(sim, iterations, has_water));
  *out = kernelsPerSubstep(schedule(sim));
  return XPBI_OK;
}

}  // extern "C"
