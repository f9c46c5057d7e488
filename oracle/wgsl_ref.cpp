// The reference's substep on the CPU — TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own WGSL entry points (web/js/shaders/simkernels.js,
// translated mechanically into oracle/_ref/xpbi_wgsl.inc by
// oracle/wgsl_ref.py) in the dispatch sequence of Simulation.encodeSubstep
// (web/js/sim.js:220-272) on the buffers of Simulation.createBuffers
// (sim.js:32-82): clearBuffer(cellTab), count, scan, scatter, the four
// reorder passes, computeL, iterations x {solveA, solveB, [pbfA, pbfB]},
// xsph, updateF, integrate, with the velA/velB ping-pong of the two bind
// groups and the final copy back into velA. Each dispatch runs
// ceil(N / 128) (or ceil(numCells / 256)) workgroups like the reference.
//
// Dispatch execution: invocations of kernels with read-modify-write atomics
// run one at a time in index order (which fixes the order WebGPU leaves
// open: within a cell the lowest index takes the highest slot); kernels with
// workgroup barriers run each workgroup's invocations as coroutines; every other
// kernel runs its invocations in parallel (they write disjoint elements).
//
// One extension beside the reference's dispatch order: pbf_iterations >= 0
// runs the PBF pair only in the first pbf_iterations iterations (the
// reference runs it in every iteration, which pbf_iterations < 0 keeps).
#include <omp.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "wgsl_rt.h"
#include "xpbi_wgsl.inc"

namespace {

using namespace wgsl;

const wgsl_ref::Entry* entry(const char* name) {
  for (const auto& e : wgsl_ref::kEntries)
    if (!std::strcmp(e.name, name)) return &e;
  return nullptr;
}

void dispatch(const wgsl_ref::Entry* e, u32 groups, int threads) {
  const u32 wg = e->wg;
  if (e->co) {
    if (e->serial) {
      for (u32 w = 0; w < groups; ++w) {
        wgsl_ref::resetWorkgroupVars();
        runWorkgroup(e->co, wg, w);
      }
      return;
    }
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
    for (long long w = 0; w < (long long)groups; ++w) {
      wgsl_ref::resetWorkgroupVars();
      runWorkgroup(e->co, wg, (u32)w);
    }
    return;
  }
  const long long total = (long long)groups * wg;
  if (e->serial) {
    for (long long g = 0; g < total; ++g)
      e->fn(vec3u((u32)g, 0u, 0u), vec3u((u32)(g % wg), 0u, 0u), vec3u((u32)(g / wg), 0u, 0u));
    return;
  }
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads)
  for (long long g = 0; g < total; ++g)
    e->fn(vec3u((u32)g, 0u, 0u), vec3u((u32)(g % wg), 0u, 0u), vec3u((u32)(g / wg), 0u, 0u));
}

}  // namespace

extern "C" {

// One or more substeps of the reference's kernels on the reference layouts
// (the same arguments as the oracle's xo_substep_f32): pos, vel and aux are
// vec4 x N, F and L are mat3x3f x N (12 floats each), params is the 256-byte
// Params block of Simulation.writeParams (sim.js:159-186) and mats the
// 8 x 16 words of writeMaterials (sim.js:84-99). sortedIdx (N) and cellTab
// (numCells) receive the last substep's permutation and cell table.
// Returns 0, or -1 if an entry point is missing, -2 on a size mismatch.
int wr_substep(const uint32_t* params, const uint32_t* mats, uint32_t n, float* pos, float* vel, float* F12,
               float* L12, float* aux, uint32_t* sortedIdx, uint32_t* cellTab, int iterations, int hasWater,
               int pbfIterations, int substeps, int threads) {
  if (threads <= 0) threads = omp_get_max_threads();
  wgsl_ref::loadUniform("P", params);
  wgsl_ref::loadUniform("MATS", mats);
  if (wgsl_ref::P.N != n) return -2;
  const uint32_t numCells = wgsl_ref::P.numCells;
  // createBuffers (sim.js:32-49): velB, and SpBuf sized for 3 vec4 per
  // particle or the scan's block sums
  std::vector<vec4f> velB(std::max<size_t>(n, 1));
  const size_t spBytes = std::max<size_t>((size_t)n * 48, ((size_t)numCells + 255) / 256 * 4 + 16);
  std::vector<vec4f> sp((spBytes + 15) / 16);
  vec4f* velA = reinterpret_cast<vec4f*>(vel);
  wgsl_ref::bindStorage("pos", pos);
  wgsl_ref::bindStorage("Fbuf", F12);
  wgsl_ref::bindStorage("Lbuf", L12);
  wgsl_ref::bindStorage("aux", aux);
  wgsl_ref::bindStorage("SpBuf", sp.data());
  wgsl_ref::bindStorage("scanAux", sp.data());
  wgsl_ref::bindStorage("cellTab", cellTab);
  wgsl_ref::bindStorage("cellTabR", cellTab);
  wgsl_ref::bindStorage("sortedIdx", sortedIdx);
  const char* names[] = {"countParticles", "scanBlocks", "scanApply", "scatter", "stagePVA", "applyPVA",
                         "stageF",         "applyF",     "computeL",  "solveA",  "solveB",   "pbfA",
                         "pbfB",           "xsph",       "updateF",   "integrate"};
  for (const char* nm : names)
    if (!entry(nm)) return -1;
  const u32 NG = (n + 127) / 128;
  const u32 NB = (numCells + 255) / 256;
  for (int s = 0; s < substeps; ++s) {
    std::memset(cellTab, 0, sizeof(uint32_t) * numCells);  // enc.clearBuffer(cellTab)
    bool flip = false;                                        // false: velA is "in"
    auto run = [&](const char* name, u32 groups, bool swap) {
      wgsl_ref::bindStorage("velIn", flip ? velB.data() : velA);
      wgsl_ref::bindStorage("velOut", flip ? velA : velB.data());
      dispatch(entry(name), groups, threads);
      if (swap) flip = !flip;
    };
    run("countParticles", NG, false);
    run("scanBlocks", NB, false);
    run("scanApply", NB, false);
    run("scatter", NG, false);
    run("stagePVA", NG, false);
    run("applyPVA", NG, false);
    run("stageF", NG, false);
    run("applyF", NG, false);
    run("computeL", NG, false);
    for (int k = 0; k < iterations; ++k) {
      run("solveA", NG, false);
      run("solveB", NG, true);
      if (hasWater && (pbfIterations < 0 || k < pbfIterations)) {
        run("pbfA", NG, false);
        run("pbfB", NG, true);
      }
    }
    run("xsph", NG, true);
    run("updateF", NG, false);
    run("integrate", NG, false);
    if (flip) std::memcpy(velA, velB.data(), sizeof(vec4f) * n);
  }
  return 0;
}

}  // extern "C"
