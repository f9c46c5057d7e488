// Cell sort for callers that cannot allocate device memory.
//
// Some hosts drive the GPU through a fixed memory budget they own: a render
// or physics engine that hands out device buffers from its own pool, a
// plugin running inside such a host, or code replayed from a CUDA graph
// captured elsewhere. They can pass us input and output buffers but cannot
// let a library call cudaMalloc at an arbitrary moment (a pool owner may
// forbid it, and a malloc inside stream capture breaks the capture). For
// them, xpbi_sort_cells_noalloc runs the uniform-grid counting sort (cell
// histogram, decoupled-lookback scan, bucket fill, crowded-bucket sort,
// deterministic ranks) with all of its scratch in one statically sized
// device array of this library, and allocates nothing.
//
// The array is a file-scope __device__ variable: every GPU that loads the
// library holds it (about 10 MB) until the process exits. Its device address
// is looked up with cudaGetSymbolAddress the first time the entry point runs
// on a device (with that device current); that first call should therefore
// happen before any stream capture. All calls share the array and it keeps
// the last call's contents, so every call clears what must start at zero, and
// calls whose work overlaps on the GPU (different streams, or different host
// threads on one device) race on it: serialise them.
//
// The prefix scan's look-back waits are bounded; one that runs out raises an
// error word inside the same array instead of the sort's outputs telling
// anything. xpbi_sort_cells_noalloc_status synchronises the caller's stream
// and reports (and clears) that word, so a caller learns of an expired wait
// without any allocation. The next sort call clears the word itself, so the
// status belongs to the last call made before it.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "xpbi.h"
#include "xpbi_internal.h"

namespace xpbi {
int setError(int code, const std::string& msg);
uint32_t launch_bigcells(const Bufs& b, uint32_t* scratch, cudaStream_t st);
}  // namespace xpbi

using namespace xpbi;

namespace {

constexpr uint32_t kMaxParticles = XPBI_NOALLOC_MAX_PARTICLES;
constexpr uint32_t kMaxCells = XPBI_NOALLOC_MAX_CELLS;
constexpr uint32_t kMaxTiles = (kMaxCells + 1 + 4095) / 4096;

// Scratch layout in 4-byte words (each region 64-word aligned).
constexpr uint32_t al(uint32_t w) { return (w + 63u) & ~63u; }
constexpr uint32_t wKey = 0;
constexpr uint32_t wTmp = wKey + al(kMaxParticles);
constexpr uint32_t wCursor = wTmp + al(kMaxParticles);
constexpr uint32_t wBigList = wCursor + al(kMaxCells + 4);
constexpr uint32_t wBigScratch = wBigList + al(kMaxParticles / 64 + 2);
constexpr uint32_t wCtl = wBigScratch + al(2 * kMaxParticles);        // ticket, count, tile descriptors (u64)
constexpr uint32_t wScene = wCtl + al(2 * (kMaxTiles + 1));
constexpr uint32_t wMats = wScene + al((sizeof(SceneDev) + 3) / 4);
constexpr uint32_t wCellWater = wMats + al((kMaxMats * sizeof(MatDev) + 3) / 4);
constexpr uint32_t wErr = wCellWater + al(kMaxCells / 4 + 4);
constexpr uint32_t wProbe = wErr + 64;  // a descriptor nothing publishes (xpbi_test_noalloc_wait_expiry)
constexpr uint32_t kWords = wProbe + 64;

static __device__ __align__(256) uint32_t g_sortScratch[kWords];

constexpr int kMaxDevices = 64;
std::mutex g_lock;
uint32_t* g_addr[kMaxDevices] = {nullptr};

// Deterministic slot of every bucket member (same rule as the substep's
// reorder): bucket start + number of members with a larger index; buckets
// above `big` members were already sorted in place.
__global__ void k_rank_only(const uint32_t* __restrict__ tmp, const uint32_t* __restrict__ key,
                            const uint32_t* __restrict__ cellStart, uint32_t n, uint32_t big,
                            uint32_t* __restrict__ sortedIdx) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t i = tmp[p];
  const uint32_t c = key[i];
  const uint32_t s0 = cellStart[c], s1 = cellStart[c + 1];
  uint32_t s = p;
  if (s1 - s0 <= big) {
    uint32_t rank = 0;
    for (uint32_t q = s0; q < s1; ++q) rank += (tmp[q] > i) ? 1u : 0u;
    s = s0 + rank;
  }
  sortedIdx[s] = i;
}

// Writes the grid description, clears the material table (no material is
// water, so no cell is flagged) and the error word.
__global__ void k_setup(SceneDev sd, SceneDev* scene, uint32_t* matWords, uint32_t nMatWords, int* err) {
  if (threadIdx.x == 0) {
    *scene = sd;
    *err = 0;
  }
  for (uint32_t w = threadIdx.x; w < nMatWords; w += blockDim.x) matWords[w] = 0u;
}

int scratchAddress(uint32_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return setError(XPBI_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return setError(XPBI_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> g(g_lock);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sortScratch);
    if (e != cudaSuccess || !p)
      return setError(XPBI_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_addr[dev] = static_cast<uint32_t*>(p);
  }
  *out = g_addr[dev];
  return XPBI_OK;
}

}  // namespace

extern "C" int xpbi_sort_cells_noalloc(const float* pos4, uint32_t n, const float origin[3], float cell_size,
                                       const int32_t dims[3], uint32_t* cell_start, uint32_t* sorted_idx,
                                       void* cuda_stream) {
  if (!pos4 || !origin || !dims || !cell_start || !sorted_idx)
    return setError(XPBI_ERR_INVALID, "NULL argument");
  if ((reinterpret_cast<uintptr_t>(pos4) & 15u) || (reinterpret_cast<uintptr_t>(cell_start) & 15u) ||
      (reinterpret_cast<uintptr_t>(sorted_idx) & 3u))
    return setError(XPBI_ERR_INVALID, "pos4 and cell_start must be 16-byte aligned, sorted_idx 4-byte aligned");
  if (n == 0 || n > kMaxParticles)
    return setError(XPBI_ERR_INVALID, "particle count must be 1.." + std::to_string(kMaxParticles) +
                                          " for the allocation-free sort");
  if (!(cell_size > 0.f)) return setError(XPBI_ERR_INVALID, "cell_size must be positive");
  for (int k = 0; k < 3; ++k)
    if (dims[k] < 1) return setError(XPBI_ERR_INVALID, "grid dimensions must be positive");
  // checked after every factor: the running product stays <= kMaxCells
  // (2^20) before each multiplication by a factor < 2^31, so it cannot wrap
  uint64_t cells = 1;
  for (int k = 0; k < 3; ++k) {
    cells *= (uint64_t)dims[k];
    if (cells > kMaxCells)
      return setError(XPBI_ERR_INVALID, "grid has more than " + std::to_string(kMaxCells) +
                                            " cells, the allocation-free sort's limit");
  }
  uint32_t* base = nullptr;
  int rc = scratchAddress(&base);
  if (rc != XPBI_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);

  SceneDev sd;
  std::memset(&sd, 0, sizeof(sd));
  for (int k = 0; k < 3; ++k) {
    sd.origin[k] = origin[k];
    sd.dims[k] = dims[k];
  }
  sd.cs = cell_size;
  sd.numCells = (uint32_t)cells;
  sd.n = n;
  Bufs b;
  std::memset(&b, 0, sizeof(b));
  b.pos = const_cast<float4*>(reinterpret_cast<const float4*>(pos4));
  b.key = base + wKey;
  b.tmp = base + wTmp;
  b.cursor = base + wCursor;
  b.cellStart = cell_start;
  b.bigList = base + wBigList;
  b.tileTicket = base + wCtl;
  b.bigCount = base + wCtl + 1;
  b.tileStatus = reinterpret_cast<unsigned long long*>(base + wCtl) + 1;
  b.scenes = reinterpret_cast<SceneDev*>(base + wScene);
  b.mats = reinterpret_cast<MatDev*>(base + wMats);  // zeroed: no material is water
  b.cellWater = reinterpret_cast<uint8_t*>(base + wCellWater);
  b.err = reinterpret_cast<int*>(base + wErr);
  b.N = n;
  b.C = (uint32_t)cells;
  b.S = 1;
  b.scanTiles = scan_tiles(b.C);

  k_setup<<<1, 128, 0, st>>>(sd, b.scenes, base + wMats, (uint32_t)((kMaxMats * sizeof(MatDev) + 3) / 4), b.err);
  launch_count(b, st);    // clears the cell counters and water flags first
  launch_scan(b, st);     // clears the look-back descriptors first
  launch_scatter(b, st);
  const uint32_t big = launch_bigcells(b, base + wBigScratch, st);
  k_rank_only<<<(n + 255) / 256, 256, 0, st>>>(b.tmp, b.key, b.cellStart, n, big, sorted_idx);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return setError(XPBI_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return XPBI_OK;
}

extern "C" int xpbi_sort_cells_noalloc_status(void* cuda_stream) {
  uint32_t* base = nullptr;
  int rc = scratchAddress(&base);
  if (rc != XPBI_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  int err = 0;
  cudaError_t e = cudaMemcpyAsync(&err, base + wErr, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return setError(XPBI_ERR_CUDA, std::string("status read: ") + cudaGetErrorString(e));
  if (err == 0) return XPBI_OK;
  e = cudaMemsetAsync(base + wErr, 0, sizeof(int), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return setError(XPBI_ERR_CUDA, std::string("status clear: ") + cudaGetErrorString(e));
  return setError(XPBI_ERR_DEVICE, "allocation-free sort: device error word 0x" + [&] {
    char t[16];
    std::snprintf(t, sizeof(t), "%x", (unsigned)err);
    return std::string(t);
  }() + " (bounded look-back wait expired; cell_start and sorted_idx are not valid)");
}

extern "C" int xpbi_test_noalloc_wait_expiry(uint32_t polls, void* cuda_stream) {
  if (polls < 1u || polls > (1u << 20)) return setError(XPBI_ERR_INVALID, "polls must be 1..1048576");
  uint32_t* base = nullptr;
  int rc = scratchAddress(&base);
  if (rc != XPBI_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  Bufs b;
  std::memset(&b, 0, sizeof(b));
  b.err = reinterpret_cast<int*>(base + wErr);
  unsigned long long* probe = reinterpret_cast<unsigned long long*>(base + wProbe);
  cudaError_t e = cudaMemsetAsync(probe, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return setError(XPBI_ERR_CUDA, std::string("probe clear: ") + cudaGetErrorString(e));
  launch_wait_expiry(b, probe, polls, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return setError(XPBI_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return XPBI_OK;
}
