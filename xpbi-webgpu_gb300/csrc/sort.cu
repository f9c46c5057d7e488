// Uniform-grid counting sort and physical reorder into cell order.
//
// Replaces clearBuffer + countParticles + scanBlocks + scanApply + scatter +
// stagePVA/applyPVA/stageF/applyF (web/js/shaders/simkernels.js:78-186,
// dispatched by web/js/sim.js:223-236) with:
//   k_count    cell key per particle + warp-aggregated histogram atomics
//   k_scan     single-pass decoupled-lookback exclusive scan of the histogram
//   k_fill     warp-aggregated slot reservation: each cell's members land in
//              its bucket in arbitrary order
//   k_bigcells deterministic sort of crowded buckets (bounded cost)
//   k_reorder  final slot = bucket start + number of bucket members with a
//              larger previous index, then moves pos/vel/F/state into the
//              slot with the scatter pass's predictor fused in
// The final slot rule reproduces the reference's atomicSub scatter executed
// in invocation order: within a cell, particles are listed by descending
// previous index. Counts, cell starts and the permutation are therefore
// deterministic and bit-identical to that serial order.
#include "xpbi_math.cuh"

namespace xpbi {

namespace {

constexpr int kThreads = 256;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr uint32_t kBigCell = 64u;          // buckets above this use k_bigcells
constexpr uint32_t kSmemSortCap = 8192u;    // bitonic in shared memory up to this size
constexpr uint32_t kLookbackSpinLimit = 1u << 22;
constexpr int kBigThreads = 256;
constexpr unsigned kBigGrid = 152;

__device__ __forceinline__ uint32_t sceneOfSlot(const Bufs& b, uint32_t i) {
  return b.S > 1 ? (uint32_t)b.sceneOf[i] : 0u;
}

__device__ __forceinline__ uint32_t cellKey(const SceneDev& S, float4 p) {
  I3 c = cellCoord(S, v3(p.x, p.y, p.z));
  return S.cellBase + cellIndex(S, c.x, c.y, c.z);
}

// cursor[] was cleared before this launch; on exit it holds cell counts.
__global__ void __launch_bounds__(kThreads) k_count(Bufs b) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool active = i < b.N;
  uint32_t key = 0;
  if (active) {
    const SceneDev& S = b.scenes[sceneOfSlot(b, i)];
    const float4 p = b.pos[i];
    key = cellKey(S, p);
    b.key[i] = key;
    uint32_t mi = 0u;
    if (p.w > 0.f) mi = min((uint32_t)p.w, 7u);
    if (b.mats[S.matBase + mi].kind == kKindWater) b.cellWater[key] = 1u;
  }
  unsigned mask = __ballot_sync(0xffffffffu, active);
  if (!active) return;
  unsigned peers = __match_any_sync(mask, key);
  int lane = threadIdx.x & 31;
  if (lane == __ffs(peers) - 1) atomicAdd(&b.cursor[key], (uint32_t)__popc(peers));
}

// Bounded wait for a look-back descriptor: polls `slot` until its flag
// (high word) is nonzero and returns the descriptor; after `polls` empty
// polls it raises kErrLookback in the error word and returns 0 (no flag),
// and the caller goes on. Nothing waits without a limit.
__device__ __forceinline__ unsigned long long waitDescriptor(const volatile unsigned long long* slot,
                                                             uint32_t polls, int* err) {
  for (uint32_t spins = 0;; ++spins) {
    const unsigned long long w64 = *slot;
    if ((uint32_t)(w64 >> 32) != 0u) return w64;
    if (spins >= polls) {
      atomicOr(err, kErrLookback);
      return 0ull;
    }
    __nanosleep(64);
  }
}

// Exclusive scan of the C counts (plus one zero item, whose prefix is the
// N sentinel) into cellStart[0..C] and cursor[0..C-1]. Tiles take a ticket
// in launch order and look back over earlier tiles' descriptors; a tile only
// waits on tiles holding smaller tickets, which are already running. Each
// wait is bounded: on expiry the error word is raised and the tile goes on.
__global__ void __launch_bounds__(kScanThreads) k_scan(Bufs b) {
  __shared__ uint32_t s_tile, s_excl;
  __shared__ uint32_t s_warp[kScanThreads / 32];
  if (threadIdx.x == 0) s_tile = atomicAdd(b.tileTicket, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t items = b.C + 1;
  const uint32_t base = tile * kScanTile + threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  if (base + kScanItems <= b.C) {
    const uint4* src = reinterpret_cast<const uint4*>(b.cursor + base);
#pragma unroll
    for (int k = 0; k < kScanItems / 4; ++k) {
      uint4 q = src[k];
      v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) v[k] = (base + k < b.C) ? b.cursor[base + k] : 0u;
  }
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    sum += v[k];
    if (v[k] > kBigCell) b.bigList[atomicAdd(b.bigCount, 1u)] = base + k;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = sum;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    uint32_t n = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += n;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kScanThreads / 32 ? s_warp[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      uint32_t n = __shfl_up_sync(0xffffffffu, wi, off);
      if (lane >= off) wi += n;
    }
    if (lane < kScanThreads / 32) s_warp[lane] = wi - w;  // exclusive warp offsets
    if (lane == kScanThreads / 32 - 1) {
      const uint32_t agg = wi;  // tile aggregate
      volatile unsigned long long* status = b.tileStatus;
      uint32_t excl = 0;
      if (tile == 0) {
        atomicExch(b.tileStatus + tile, (2ull << 32) | agg);
      } else {
        atomicExch(b.tileStatus + tile, (1ull << 32) | agg);
        int pred = (int)tile - 1;
        while (pred >= 0) {
          const unsigned long long w64 = waitDescriptor(status + pred, kLookbackSpinLimit, b.err);
          const uint32_t flag = (uint32_t)(w64 >> 32);
          if (flag == 0u) break;  // the wait expired (error word raised)
          excl += (uint32_t)w64;
          if (flag == 2u) break;
          --pred;
        }
        __threadfence();
        atomicExch(b.tileStatus + tile, (2ull << 32) | (excl + agg));
      }
      s_excl = excl;
    }
  }
  __syncthreads();
  uint32_t run = s_excl + s_warp[warp] + (incl - sum);
  uint32_t out[kScanItems];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) { out[k] = run; run += v[k]; }
  if (base + kScanItems <= b.C) {
    uint4* d0 = reinterpret_cast<uint4*>(b.cellStart + base);
    uint4* d1 = reinterpret_cast<uint4*>(b.cursor + base);
#pragma unroll
    for (int k = 0; k < kScanItems / 4; ++k) {
      uint4 q = make_uint4(out[4 * k], out[4 * k + 1], out[4 * k + 2], out[4 * k + 3]);
      d0[k] = q;
      d1[k] = q;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      uint32_t idx = base + k;
      if (idx < items) b.cellStart[idx] = out[k];
      if (idx < b.C) b.cursor[idx] = out[k];
    }
  }
}

// Unordered bucket fill: tmp[cellStart[key] .. +count) receives the members.
__global__ void __launch_bounds__(kThreads) k_fill(Bufs b) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool active = i < b.N;
  uint32_t key = active ? b.key[i] : 0u;
  unsigned mask = __ballot_sync(0xffffffffu, active);
  if (!active) return;
  unsigned peers = __match_any_sync(mask, key);
  int lane = threadIdx.x & 31;
  int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(&b.cursor[key], (uint32_t)__popc(peers));
  base = __shfl_sync(mask, base, leader);
  uint32_t rank = __popc(peers & ((1u << lane) - 1u));
  b.tmp[base + rank] = i;
}

// Buckets with more than kBigCell members (listed by k_scan) are sorted
// here, descending, by one CTA each: a bitonic network on ~index ascending, in
// shared memory up to kSmemSortCap entries, otherwise in the scratch region
// [2*start, 2*start + 2*len) of `scratch`, which is disjoint between buckets.
// Cost is O(L log^2 L) per bucket, so even a pile-up of every particle in one
// cell stays bounded. With no crowded cell every CTA exits at once.
__device__ __forceinline__ void bitonic_sort_asc(uint32_t* a, uint32_t n2) {
  for (uint32_t size = 2; size <= n2; size <<= 1) {
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t t = threadIdx.x; t < n2 / 2; t += blockDim.x) {
        uint32_t lo = 2 * stride * (t / stride) + (t % stride);
        uint32_t hi = lo + stride;
        bool up = ((lo & size) == 0);
        uint32_t x = a[lo], y = a[hi];
        if ((x > y) == up) { a[lo] = y; a[hi] = x; }
      }
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(kBigThreads) k_bigcells(Bufs b, uint32_t* scratch) {
  extern __shared__ uint32_t sm[];
  const uint32_t nBig = *b.bigCount;
  for (uint32_t j = blockIdx.x; j < nBig; j += gridDim.x) {
    uint32_t cell = b.bigList[j];
    uint32_t s0 = b.cellStart[cell], len = b.cellStart[cell + 1] - s0;
    uint32_t n2 = 1;
    while (n2 < len) n2 <<= 1;
    uint32_t* a = n2 <= kSmemSortCap ? sm : scratch + 2ull * s0;
    for (uint32_t q = threadIdx.x; q < n2; q += blockDim.x) a[q] = q < len ? ~b.tmp[s0 + q] : 0xffffffffu;
    __syncthreads();
    bitonic_sort_asc(a, n2);
    for (uint32_t q = threadIdx.x; q < len; q += blockDim.x) b.tmp[s0 + q] = ~a[q];
    __syncthreads();
  }
}

// Final slot + physical reorder with the scatter pass's predictor fused in
// (simkernels.js:137-146 and 154-186).
__global__ void __launch_bounds__(kThreads) k_reorder(Bufs b, int keepLam) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  // both slots of the substep's largest-solid-displacement ring start at 0
  for (uint32_t q = p; q < 2u * b.S; q += gridDim.x * blockDim.x) b.solidDisp[q] = 0u;
  if (p >= b.N) return;
  uint32_t i = b.tmp[p];
  uint32_t key = b.key[i];
  uint32_t s0 = b.cellStart[key], s1 = b.cellStart[key + 1];
  uint32_t s;
  if (s1 - s0 > kBigCell) {
    s = p;  // bucket already sorted by k_bigcells
  } else {
    uint32_t rank = 0;
    for (uint32_t q = s0; q < s1; ++q) rank += (b.tmp[q] > i) ? 1u : 0u;
    s = s0 + rank;
  }
  b.sortedIdx[s] = i;
  const SceneDev& S = b.scenes[sceneOfSlot(b, i)];
  // sorted records carry the water flag in the sign bit of pos.w (>= 0)
  const float4 pp = b.pos[i];
  uint32_t mi = 0u;
  if (pp.w > 0.f) mi = min((uint32_t)pp.w, 7u);
  const bool water = b.mats[S.matBase + mi].kind == kKindWater;
  b.posS[s] = make_float4(pp.x, pp.y, pp.z, water ? -pp.w : pp.w);
  M3 F = loadM(b.F, b.N, i);
  storeM(b.FS, b.N, s, F);
  float Vn = S.V0 * clampf(det(F), 0.1f, 10.f);
  float4 v = b.vel[i];
  V3 g = v3(S.grav[0], S.grav[1], S.grav[2]);
  V3 vn = xyz(v) + g * S.dt;
  b.velS[0][s] = make_float4(vn.x, vn.y, vn.z, Vn);
  b.stateS[s] = b.state[i];
  b.lam[s] = 0.f;
  if (keepLam) b.lamPrev[s] = b.lamOut[i];
}

inline unsigned grid(uint32_t n, int t) { return (unsigned)((n + t - 1) / t); }

// Test hook: the scan's bounded wait on a descriptor nothing publishes
// (`slot` stays zero), so the wait expires after `polls` polls and raises
// the error word the host reads — the failure path of the look-back without
// a fault. One thread.
__global__ void k_wait_expiry(Bufs b, const unsigned long long* slot, uint32_t polls) {
  waitDescriptor(slot, polls, b.err);
}

}  // namespace

uint32_t scan_tiles(uint32_t cells) { return (cells + 1 + kScanTile - 1) / kScanTile; }

void launch_count(const Bufs& b, cudaStream_t st) {
  cudaMemsetAsync(b.cursor, 0, sizeof(uint32_t) * b.C, st);
  cudaMemsetAsync(b.cellWater, 0, b.C, st);
  k_count<<<grid(b.N, kThreads), kThreads, 0, st>>>(b);
}
void launch_wait_expiry(const Bufs& b, const unsigned long long* slot, uint32_t polls, cudaStream_t st) {
  k_wait_expiry<<<1, 1, 0, st>>>(b, slot, polls);
}
void launch_scan(const Bufs& b, cudaStream_t st) {
  // ticket, crowded-cell count and tile descriptors are contiguous: one
  // memset resets all three
  cudaMemsetAsync(b.tileTicket, 0, sizeof(unsigned long long) * (b.scanTiles + 1), st);
  k_scan<<<b.scanTiles, kScanThreads, 0, st>>>(b);
}
void launch_scatter(const Bufs& b, cudaStream_t st) {
  k_fill<<<grid(b.N, kThreads), kThreads, 0, st>>>(b);
}
void launch_reorder(const Bufs& b, bool keepLam, cudaStream_t st) {
  // scratch for buckets too large for shared memory lives in the Sp buffer
  // (16 floats per particle >= 2 words per particle), unused until solveA
  uint32_t* scratch = reinterpret_cast<uint32_t*>(b.Sp);
  k_bigcells<<<kBigGrid, kBigThreads, kSmemSortCap * sizeof(uint32_t), st>>>(b, scratch);
  k_reorder<<<grid(b.N, kThreads), kThreads, 0, st>>>(b, keepLam ? 1 : 0);
}

// The crowded-bucket sort alone, with caller-provided scratch of at least
// 2N words; buckets above the returned member count are left sorted.
uint32_t launch_bigcells(const Bufs& b, uint32_t* scratch, cudaStream_t st) {
  k_bigcells<<<kBigGrid, kBigThreads, kSmemSortCap * sizeof(uint32_t), st>>>(b, scratch);
  return kBigCell;
}

}  // namespace xpbi
