// Headless renderer: the camera and frame parameters of one image.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace xpbi {

struct RenderParams {
  float view[16];      // column-major (mat4LookAt, main.js:33-43)
  float proj[16];      // column-major, depth in [0, 1] (mat4Persp, main.js:44-52)
  float viewProj[16];  // proj * view
  float eye[3];
  float lightDir[3];   // world, normalised
  float particleRadius;
  float groundY;
  float nearZ;
  float boxMin[3], boxMax[3];
  int width, height;
  int drawGround, drawBox;
  int maxPixelsPerParticle;  // particles covering more pixels are skipped
};

// Rasterises one frame of n particles (current arrays, pos.w = material +
// colour seed) into img (width x height packed depth/colour words) and
// resolves its colours into rgba (RGBA8 per pixel, row 0 at the top).
void render_frame(const RenderParams& P, const float4* pos, const float4* vel, const uint32_t* matWords, uint32_t n,
                  unsigned long long* img, uint32_t* rgba, cudaStream_t st);

}  // namespace xpbi
