// Internal types shared by the host API and the kernels of libxpbi.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace xpbi {

constexpr int kMaxMats = 8;            // simkernels.js:19
constexpr uint32_t kRowCap = 384u;     // simkernels.js:73
constexpr uint32_t kKindSnow = 5u;
constexpr uint32_t kKindWater = 6u;

constexpr uint32_t kNbrCap = 64u;      // neighbour-list capacity per particle
constexpr int kSolveAVariants = 6;      // launch-shape variants (autotuner): block size, register cap
constexpr int kSolveBVariants = 5;
// Lanes per slot of solveA / solveB by the handle's solid particle count:
// four up to 24k solids, two up to 48k, else one (measured on sand columns,
// dam breaches of 8k-120k solids and the 113k-solid snowball)
constexpr uint64_t kFourLaneSolids = 24576;
constexpr uint64_t kTwoLaneSolids = 49152;
constexpr int kResidBlocks = 256;      // at most this many partial sums of the residual per scene
constexpr int kMaxResid = 129;         // residual slots per scene (iterations + 1)
constexpr int kFeat = 16;              // network features per particle

// solveA flags
constexpr int kTrackResid = 1;         // write per-particle residuals
constexpr int kWarm = 2;               // iteration 0 starts from lamWarm
constexpr int kMeasureOnly = 4;        // residual only: no multiplier / impulse update
constexpr int kStoredC = 8;            // iteration 0 reads the constraint computeL stored (features)
// active set (solveA / solveB / pbfB flags)
constexpr int kMarkMoved = 16;         // a slot whose velocity changed marks itself (and, if solid, its solid
                                       // neighbours) as changed for the next iteration
constexpr int kActive = 32;            // iteration k >= 1 visits only the slots whose inputs changed
constexpr int kRerun = 64;             // the plain re-solve of the scenes an early-stopped solve failed
constexpr int kInPlace = 128;          // solveB of the active set: in place, one lane per slot
constexpr int kIterDevice = -1000000;  // a kernel's iteration argument: read it from Bufs::kIter (device loop)
constexpr uint32_t kNbrOverflow = 0xffffffffu;
constexpr uint32_t kWaterBit = 0x80000000u;

// Device error word bits.
constexpr int kErrLookback = 1;        // decoupled look-back wait expired

// One scene's uniforms plus constants derived from them on the host. Every
// derived constant is formed in f32 with the operation order of the per-call
// WGSL expression it replaces, so it is bit-identical to recomputing it.
struct SceneDev {
  float origin[3];
  float cs;                 // cell size = support
  int dims[3];
  uint32_t numCells;
  uint32_t cellBase;        // first global cell of this scene
  uint32_t pBase;           // first global particle of this scene
  uint32_t n;               // particles of this scene
  uint32_t matBase;         // first global material (scene * 8)
  float dmin[3];
  float dt;
  float dmax[3];
  float h;
  float grav[3];
  float support;
  float colPos[3];
  float colR;
  float colVel[3];
  float colActive;
  float V0, xsphC, omega, pbfEps;
  float sCorrK, contactOmega, kDamp, support2;
  float sigW;               // 21 / (16 pi h^3)            common.js:67
  float poly6C;             // 315 / (64 pi H^9)           common.js:86
  float spikyC;             // -45 / (pi H^6)              common.js:93
  float w00;                // poly6(0)                    simkernels.js:416
  float w0;                 // poly6(0.2 H)                simkernels.js:465
  float alphaT;             // (1/V0)/(dt dt)              simkernels.js:302
  float minD;               // 0.75 h                      simkernels.js:333
  float vmaxCFL;            // 0.45 support / dt           simkernels.js:535
  float dvCap;              // 0.2 support / dt            simkernels.js:361
  float invH;               // 1 / h
  float invW0;              // 1 / max(w0, 1e-12)          simkernels.js:466
  int iterations;           // XPBI Jacobi iterations this substep (an early-stopped solve's cap)
  int pbfIterations;        // PBF passes (first k iterations)
  int pbfUntil;             // iterations k < pbfUntil run a PBF pass (the scene's own schedule)
  int plainIterations;      // the scene's own iteration count (the plain re-solve's budget)
  int hasWater;
  float residTol;           // early stop at |r_k| <= residTol |C(v_pred)|; <= 0: never
  float residTolC;          // ... and |contact_k| <= residTolC |contact_0|
  float waterMpd;           // mass / density of the scene's one water material; 0: none or several
  uint32_t nSolid;          // solid particles of the scene
  float asShare;            // active set: share of the residual budget settled particles may hold (0: off)
};

struct MatDev {
  float mu, lam, density;
  uint32_t kind;
  float p0, p1, p2, p3;
  float boundFriction, mass;
  float massPerDensity;     // mass / density (host f32, the same IEEE quotient as on the device)
  float pad;
};

// Device buffers of one handle. "Current" arrays hold the state between
// substeps in the cell order of the last substep; the "sorted" arrays are the
// substep's working copies written by the reorder.
struct Bufs {
  float4* pos;          // [N] current positions, w = material + seed
  float4* vel;          // [N] current velocities, w = V^n
  float* F;             // [9][N] current F, plane (3c+r) holds F[c][r]
  float* state;         // [N] current plastic state
  float4* posS;         // [N] sorted positions
  float4* velS[2];      // [N] Jacobi ping-pong velocities
  float* FS;            // [9][N] sorted F
  float* stateS;        // [N] sorted plastic state
  float* L;             // [9][N] kernel-gradient correction
  float4* sgP;          // [3][N] a solid's velocity-free sums over its solid neighbours (computeL):
                        //   (sum V g, count), (P00, P11, P22, P01), (P02, P12, -, -), P = sum V^2/m g g^T
  float* lam;           // [N] XPBI multiplier
  float* pbfLam;        // [N] PBF multiplier
  float4* Sp;           // [4][N] solveB neighbour record planes: dlam G L columns (x, y, z in .w), x + dt v, mass
  float4* SpSelf;       // [N] own dv of the constraint update (sgrad * dlam)
  uint32_t* key;        // [N] global cell of each current particle
  uint32_t* tmp;        // [N] unordered cell-bucket fill
  uint32_t* sortedIdx;  // [N] global previous index of each sorted slot
  uint32_t* cursor;     // [C] per-cell fill cursor
  uint32_t* cellStart;  // [C+1] exclusive cell starts, sentinel = N
  uint8_t* cellWater;   // [C] 1 if the cell holds a water particle this substep
  uint32_t* tileTicket;            // word 0 of the scan control block
  uint32_t* bigCount;              // word 1: crowded cells found by the scan
  unsigned long long* tileStatus;  // [tiles] look-back descriptors (after the two words)
  uint32_t* bigList;               // [N/64 + 2] crowded cells (> 64 members)
  uint16_t* sceneOf;    // [N] scene of each particle slot (static)
  uint32_t* nbr;        // [N][kNbrCap] in-support neighbours, stencil order: index | water << 31
  uint32_t* nbrCount;   // [N] list length, kNbrOverflow if it did not fit
  uint32_t* nbrP;       // [N][kNbrCap] predicted-position neighbours of the current PBF pass
  uint32_t* nbrPCount;  // [N]
  float4* xc;           // [N] predicted positions x + dt v of the current PBF pass, w = pos.w
  float4* pbfRec;       // [N] the same predicted position with the pass's PBF multiplier in .w (written by pbfA)
  // solver instrumentation and warm start
  float* lamOut;        // [N] final multiplier of the last substep, current order
  float* lamPrev;       // [N] the same, carried into this substep's sorted order
  float* lamWarm;       // [N] warm-start multiplier for iteration 0 (sorted)
  float* feat;          // [N][16] network features at iteration 0 (sorted)
  float4* cons0;        // [4][N] iteration 0's constraint stored by computeL: C, denom, cdot, sgrad, GL
  float* netOut;        // [N] network output
  float* rr;            // [N] squared constraint residual of the current iteration
  float* c0sq;          // [N] squared constraint value at the predicted velocities
  float* rc;            // [N] squared contact correction of the current iteration
  uint32_t* solidDisp;  // [2][S] float bits: largest dt |v| of a scene's solids entering iteration k (slot k & 1)
  double* residPart;    // [S][kResidBlocks][4] partial sums
  uint32_t* residTicket; // [S] blocks of the residual reduction done (0 between launches)
  double* resid;        // [S][kMaxResid] residual norm^2 per iteration (last slot: after the last)
  double* residC;       // [S][kMaxResid] contact residual norm^2, same slots
  double* c0;           // [S] |C(v_pred)|^2
  double* cc0;          // [S] contact residual^2 entering iteration 0
  int* done;            // [S] converged: later iterations skip
  // active set: per-slot flags (bytes, set by plain stores of 1 from any thread)
  uint8_t* dirty[2];    // [N] by iteration parity: the slot's constraint or contact inputs changed
  uint8_t* bmark;       // [N] a solid neighbour received an impulse in this iteration's solveA
  uint8_t* imp;         // [N] k + 1 if the slot took an impulse in iteration k (solveB gathers its record only
                        //   then); cleared each substep
  uint32_t* listA;      // [N] solid slots solveA re-evaluates this iteration (compacted)
  uint32_t* listB;      // [N] slots solveB updates this iteration (compacted)
  float* thr;           // [S][3] squared per-slot thresholds: settled constraint, settled contact, and the
                        //   velocity change below which a slot does not count as moved
  float* dv0sq;         // [N] |velocity change|^2 of each solid in iteration 0 (its scale for the last one)
  uint32_t* actA;       // [kMaxResid] solid slots solveA evaluated, per iteration (listA's length)
  uint32_t* actB;       // [kMaxResid] slots solveB updated, per iteration (listB's length)
  int* kIter;           // [1] iteration of the device loop's current pass (kIterDevice)
  float4* vel0;         // [N] velocities entering iteration 0 (the plain re-solve starts from them)
  int* rerun;           // [S] 1: the early-stopped solve missed its tolerances, re-solved plainly
  int* itersUsed;       // [S] iterations whose update was applied
  void* netBlob;        // packed network weights
  SceneDev* scenes;     // [S]
  MatDev* mats;         // [S * 8]
  int* err;             // [1] device error word
  unsigned long long* waitProbe;  // [1] a descriptor nothing publishes (xpbi_test_wait_expiry)
  uint32_t N, C, S;
  uint32_t maxSceneN;   // particles of the largest scene
  uint32_t scanTiles;
};

// ---- launchers (sort.cu) ----
void launch_count(const Bufs& b, cudaStream_t st);
void launch_scan(const Bufs& b, cudaStream_t st);
void launch_wait_expiry(const Bufs& b, const unsigned long long* slot, uint32_t polls, cudaStream_t st);
void launch_scatter(const Bufs& b, cudaStream_t st);
void launch_reorder(const Bufs& b, bool keepLam, cudaStream_t st);
void launch_warm_from_prev(const Bufs& b, cudaStream_t st);
uint32_t scan_tiles(uint32_t cells);

// ---- launchers (solve.cu) ----
// sums: also form the solids' velocity-free constraint sums (sgP);
// features: also iteration 0's constraint (cons0) and the network features
void launch_computeL(const Bufs& b, bool sums, bool features, cudaStream_t st);
// the water particles' L of the last substep (computeL forms the solids' only)
void launch_computeL_water(const Bufs& b, cudaStream_t st);
void launch_solveA(const Bufs& b, int k, const float4* velIn, int flags, int variant, int lanes, cudaStream_t st);
void launch_warm_from_net(const Bufs& b, cudaStream_t st);
void launch_resid_reduce(const Bufs& b, int k, bool warm, cudaStream_t st);
void launch_keep_lambda(const Bufs& b, cudaStream_t st);

// ---- network (mlp.cu) ----
size_t mlp_blob_bytes();
void mlp_pack(const float* dParams, void* dBlob, cudaStream_t st);
// skipZero: tiles whose 128 feature rows are all zero output 0 without running the network
cudaError_t mlp_forward(const float* dX, uint32_t rows, const void* dBlob, float* dY, float* dZ, int* dErr,
                        cudaStream_t st, bool skipZero = false);
void launch_solveB(const Bufs& b, int k, const float4* velIn, float4* velOut, bool writeXc, int flags, int variant,
                   int lanes, cudaStream_t st);
void launch_pbfA(const Bufs& b, int k, const float4* velIn, int flags, cudaStream_t st);
// the plain re-solve: judge marks the scenes whose early-stopped solve did
// not stop (sets the graph's condition when setCond), restore resets their
// velocities in `vel` to vel0, copy moves every slot's velocity src -> dst
void launch_judge(const Bufs& b, cudaGraphConditionalHandle h, bool setCond, cudaStream_t st);
void launch_restore(const Bufs& b, float4* vel, cudaStream_t st);
void launch_copy_vel(const Bufs& b, const float4* src, float4* dst, cudaStream_t st);
// every slot's predicted position for pbfA from the velocities in `vel`
void launch_predict(const Bufs& b, const float4* vel, cudaStream_t st);
// active set, iterations from 2: compact the changed solids (which = 0,
// listA) or the changed and impulse-receiving slots (which = 1, listB),
// then run solveA / solveB over the list
void launch_compact(const Bufs& b, int k, int which, cudaStream_t st);
void launch_solveA_list(const Bufs& b, int k, const float4* velIn, int flags, int variant, cudaStream_t st);
void launch_solveB_list(const Bufs& b, int k, float4* vel, int flags, int variant, cudaStream_t st);
// the device loop over an early-stopped solve's last iterations (a while
// node of the substep's graph): begin sets the iteration to k0, next
// advances it; both set the node's condition to whether any scene is still
// iterating (not stopped, below its cap)
void launch_loop_begin(const Bufs& b, int k0, cudaGraphConditionalHandle h, cudaStream_t st);
void launch_loop_next(const Bufs& b, cudaGraphConditionalHandle h, cudaStream_t st);
void launch_pbfB(const Bufs& b, int k, const float4* velIn, float4* velOut, int flags, cudaStream_t st);
void launch_xsph(const Bufs& b, const float4* velIn, float4* velOut, cudaStream_t st);
void launch_updateF_integrate(const Bufs& b, const float4* velIn, cudaStream_t st);

}  // namespace xpbi
